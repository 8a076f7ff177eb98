"""Per-node pool search (inSearch / poolSearch) on the GPU (kcna_pool_search.cu)
against the reference's own inSearch (tests/golden/ref_pool_search_*.npz) and
the oracle, and inside a build (params.refine = pool search)."""
import os
import time

import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
P = dict(K=48, L=48, S=8, R=48, iterations=5, search_L=24, nsg_R=16, search_K=48, controls=20, massq_S=8,
         angle=60.0)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("loop", [1, 2])
def test_gpu_pool_search_vs_reference(index, oracle, name, loop):
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    g = dict(np.load(os.path.join(HERE, f"ref_pool_search_{name}.npz")))
    X = z["X"].astype(np.float32)
    p = kcna.params(**P, tau=float(z["tau"]))
    index.upload(X)
    index.set_pools(z["pool_ids"], z["pool_d"], z["pool_cnt"], p)
    index.set_graph(z["link_nsg_ids"], z["link_nsg_deg"], 0)
    cc = index.pool_search(loop, p)
    pid, pd, pc = index.pools()
    assert np.array_equal(pc, g[f"loop{loop}_cnt"])
    assert np.array_equal(pid[:, :48], g[f"loop{loop}_ids"])
    n = X.shape[0]
    assert cc / (n * (n - 1) / 2) == pytest.approx(float(g[f"loop{loop}_scan"]), rel=1e-5)
    # distances: the reference's own on integer rows, the oracle's canonical chain on float rows
    if name == "c2":
        assert np.array_equal(pd[:, :48], g[f"loop{loop}_d"])
    else:
        _, od, _, _ = oracle.pool_search(X, oracle_py.params(**P, tau=float(z["tau"])), z["pool_ids"], z["pool_d"],
                                         z["pool_cnt"], z["link_nsg_ids"], z["link_nsg_deg"], loop)
        assert np.array_equal(pd[:, :48], od)


def test_gpu_pool_search_vs_oracle_c2_20k(index, oracle):
    """20k C2 rows: the GPU's own NN-descent pools and NSG link graph, loops 1-3
    run in sequence, each against the oracle from the same input."""
    X = synth.base("c2", 20000)
    kw = dict(K=100, L=100, S=12, R=100, iterations=4, search_L=40, nsg_R=32, search_K=100, step=10)
    index.upload(X)
    index.nndescent(kcna.params(**kw))
    p = kcna.params(**kw)
    index.link("nsg", p)
    gids, gdeg, _ = index.graph()
    for loop in (1, 2, 3):
        pid, pd, pc = index.pools()
        oi, od, oc, occ = oracle.pool_search(X, oracle_py.params(**kw), pid, pd, pc, gids, gdeg, loop)
        cc = index.pool_search(loop, p)
        gi2, gd2, gc2 = index.pools()
        assert np.array_equal(gc2, oc)
        assert np.array_equal(gi2, oi)
        assert np.array_equal(gd2, od)
        assert cc == occ


def test_gpu_build_with_pool_search_refinement():
    X = synth.base("c2", 50000)
    kw = dict(K=100, L=100, S=12, R=100, iterations=6, search_L=40, nsg_R=32, search_K=100, loop_i=2, recall=0.99)
    with kcna.Index(0) as ix:
        ix.upload(X)
        st1 = ix.build("nsg", kcna.params(refine=1, **kw))
        st0 = ix.build("nsg", kcna.params(**kw))
        ix.build("nsg", kcna.params(refine=1, **kw))
        t = time.perf_counter()
        ix.pool_search(3, kcna.params(**kw))
        dt = time.perf_counter() - t
    r1, r0 = st1["loop_recall"], st0["loop_recall"]
    assert st1["bridge_comps"] > 0 and st1["loops"] == 3
    assert r1[2] >= r1[0] - 1e-6 and r1[2] >= 0.99
    print(f"\npool-search refinement, 50k x 128: loop recall {r1[:3]} (BridgeView {r0[:3]}); "
          f"one pool search {1e3 * dt:.1f} ms")
