"""The CUDA path against golden outputs of the reference itself
(tests/golden/ref_*.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from fastkcna_gb300 import kcna

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
P = dict(K=48, L=48, S=8, R=48, iterations=5, search_L=24, nsg_R=16, search_K=48, controls=20, massq_S=8,
         angle=60.0)
KINDS = (("nsg", "nsg"), ("taumng", "tau"), ("alphapg", "alpha"))


def load(name):
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    z["X"] = z["X"].astype(np.float32)
    return z


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_gpu_exact_knn_vs_reference(index, name):
    z = load(name)
    index.upload(z["X"])
    gi, gd = index.knn_exact(z["knn_q"], z["knn_ids"].shape[1])
    assert np.array_equal(gi, z["knn_ids"])
    if name == "c2":
        assert np.array_equal(gd, z["knn_d"])


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("kind,tag", KINDS)
def test_gpu_prune_link_vs_reference(index, name, kind, tag):
    z = load(name)
    p = kcna.params(**P, tau=float(z["tau"]))
    index.upload(z["X"])
    index.set_pools(z["pool_ids"], z["pool_d"], z["pool_cnt"], p)
    index.prune(kind, p)
    g, deg, _ = index.graph()
    W = z[f"prune_{tag}_ids"].shape[1]
    assert np.array_equal(deg, z[f"prune_{tag}_deg"])
    assert np.array_equal(g[:, :W], z[f"prune_{tag}_ids"][:, : g.shape[1]])
    index.set_pools(z["pool_ids"], z["pool_d"], z["pool_cnt"], p)
    index.link(kind, p)
    g, deg, _ = index.graph()
    assert np.array_equal(deg, z[f"link_{tag}_deg"])
    for i in range(g.shape[0]):
        assert set(g[i, : deg[i]].tolist()) == set(z[f"link_{tag}_ids"][i, : deg[i]].tolist())


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_gpu_beam_search_vs_reference(index, name):
    z = load(name)
    index.upload(z["X"])
    index.set_graph(z["link_nsg_ids"], z["link_nsg_deg"], 0)
    bi, bd = index.search(z["bs_q"], 24, 10, z["bs_init"])
    assert np.array_equal(bi, z["bs_ids"])
    if name == "c2":
        assert np.array_equal(bd, z["bs_d"])
