"""CAGRA-style rank prune on the GPU (kcna_cagra.cu) against the reference's
own BuildCagra (tests/golden/ref_cagra_*.npz) and the oracle, including a hub
node whose reverse list is streamed through the merge kernel's best set."""
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
@pytest.mark.parametrize("k", [48, 46])
def test_gpu_cagra_vs_reference(index, name, k):
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    c = dict(np.load(os.path.join(HERE, f"ref_cagra_{name}.npz")))
    p = kcna.params(**dict(P, K=k), tau=float(z["tau"]))
    index.upload(z["X"].astype(np.float32))
    index.set_pools(z["pool_ids"], z["pool_d"], z["pool_cnt"], p)
    index.prune("cagra", p)
    g, deg, _ = index.graph()
    assert np.array_equal(deg, c[f"k{k}_deg"])
    W = c[f"k{k}_ids"].shape[1]
    assert np.array_equal(g[:, :W], c[f"k{k}_ids"])


def test_gpu_cagra_hub_and_short_pools(index, oracle):
    """Node 0 heads every other pool (in-degree ~n, above the 2,048 keys the
    merge sorts at once) and every 7th pool is cut short of K."""
    X = synth.base("c2", 6000)
    n, K = X.shape[0], 32
    kw = dict(K=K, L=K, S=8, R=32, iterations=4, search_L=24, nsg_R=16, search_K=K, controls=10)
    index.upload(X)
    index.nndescent(kcna.params(**kw))
    pid, pd, pc = index.pools()
    pid, pd, pc = pid[:, :K].copy(), pd[:, :K].copy(), np.minimum(pc, K).astype(np.uint32)
    for i in range(1, n):
        row = [j for j in pid[i, : pc[i]] if j != 0][: K - 1]
        pid[i, 0], pd[i, 0] = 0, 0.0
        pid[i, 1: 1 + len(row)] = row
        pc[i] = 1 + len(row)
    pc[::7] = np.minimum(pc[::7], K - 5)
    p = kcna.params(**kw)
    index.set_pools(pid, pd, pc, p)
    index.prune("cagra", p)
    g, deg, _ = index.graph()
    oi, _, odeg = oracle.prune(oracle_py.KCNA_CAGRA, X, oracle_py.params(**kw), pid, pd, pc, K // 2 + 1)
    assert np.array_equal(deg, odeg)
    assert np.array_equal(g[:, : K // 2 + 1], oi)
    assert (g[1:, 0] == 0).mean() > 0.5  # the hub is kept by most nodes


def test_gpu_cagra_c2_scale(index):
    """K = 64 on the pools of a 200k-row C2 NN-descent: degrees and timing."""
    X = synth.base("c2", 200_000)
    kw = dict(K=64, L=64, S=12, R=64, iterations=6, search_L=40, nsg_R=32, search_K=64)
    index.upload(X)
    index.nndescent(kcna.params(**kw))
    p = kcna.params(**kw)
    index.prune("cagra", p)  # warm
    t = time.perf_counter()
    index.prune("cagra", p)
    dt = time.perf_counter() - t
    g, deg, _ = index.graph()
    assert deg.min() >= 32 and deg.max() <= 33
    assert (g[np.arange(len(deg)), 0] < len(deg)).all()
    print(f"\nCAGRA rank prune, 200k x 128, K = 64: {1e3 * dt:.1f} ms")
