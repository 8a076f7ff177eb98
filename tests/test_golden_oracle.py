"""The oracle restatement against golden outputs of the reference itself.

tests/golden/ref_*.npz were produced by the reference's own code
(tests/golden/make_golden.py).  On the integer-valued set every distance is
exact in any summation order, so the oracle must match bit for bit; on the
float set the reference sums in an AVX lane order, so distances may differ in
the last bits while ids and edge lists must still match.
"""
import os

import numpy as np
import pytest

import oracle_py

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    z["X"] = z["X"].astype(np.float32)
    return z


P = dict(K=48, L=48, S=8, R=48, iterations=5, search_L=24, nsg_R=16, search_K=48, controls=20, massq_S=8,
         angle=60.0)
KINDS = ((1, "nsg"), (3, "tau"), (4, "alpha"))


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_exact_knn(oracle, name):
    z = load(name)
    oi, od = oracle.knn(z["X"], z["knn_q"], z["knn_ids"].shape[1])
    assert np.array_equal(oi, z["knn_ids"])
    if name == "c2":
        assert np.array_equal(od, z["knn_d"])
    else:
        np.testing.assert_allclose(od, z["knn_d"], rtol=2e-6)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("kind,tag", KINDS)
def test_prune_and_link(oracle, name, kind, tag):
    z = load(name)
    p = oracle_py.params(**P, tau=float(z["tau"]))
    W = z[f"prune_{tag}_ids"].shape[1]
    gi, _, deg = oracle.prune(kind, z["X"], p, z["pool_ids"], z["pool_d"], z["pool_cnt"], W)
    assert np.array_equal(deg, z[f"prune_{tag}_deg"])
    assert np.array_equal(gi, z[f"prune_{tag}_ids"])
    gi, _, deg = oracle.link(kind, z["X"], p, z["pool_ids"], z["pool_d"], z["pool_cnt"], W)
    assert np.array_equal(deg, z[f"link_{tag}_deg"])
    for i in range(gi.shape[0]):  # reverse-edge order follows thread timing in the reference: compare sets
        assert set(gi[i, : deg[i]].tolist()) == set(z[f"link_{tag}_ids"][i, : deg[i]].tolist())


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_beam_search(oracle, name):
    z = load(name)
    bi, bd = oracle.beam_search(z["X"], z["link_nsg_ids"], z["link_nsg_deg"], z["bs_q"], z["bs_init"], 24, 10)
    assert np.array_equal(bi, z["bs_ids"])
    if name == "c2":
        assert np.array_equal(bd, z["bs_d"])


def test_pools_are_valid_knn_pools():
    for name in ("c1", "c2"):
        z = load(name)
        for i in range(0, z["pool_ids"].shape[0], 50):
            c = z["pool_cnt"][i]
            row = z["pool_ids"][i, :c]
            assert len(set(row.tolist())) == c and i not in row
            assert np.all(np.diff(z["pool_d"][i, :c]) >= 0)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("k", [48, 46])
def test_cagra_prune(oracle, name, k):
    """CAGRA rank prune (BuildCagra) of the reference's pools, K = 48 (even
    prune_K) and K = 46 (odd prune_K: rows of prune_K + 1)."""
    z = load(name)
    c = dict(np.load(os.path.join(HERE, f"ref_cagra_{name}.npz")))
    p = oracle_py.params(**dict(P, K=k), tau=float(z["tau"]))
    gi, gd, deg = oracle.prune(oracle_py.KCNA_CAGRA, z["X"], p, z["pool_ids"], z["pool_d"], z["pool_cnt"], k // 2 + 1)
    assert np.array_equal(deg, c[f"k{k}_deg"])
    assert np.array_equal(gi, c[f"k{k}_ids"])
    if name == "c2":
        assert np.array_equal(gd, c[f"k{k}_d"])
    else:
        np.testing.assert_allclose(gd, c[f"k{k}_d"], rtol=2e-6)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("loop", [1, 2])
def test_pool_search(oracle, name, loop):
    """Per-node pool search (inSearch) of the reference's pools over its NSG
    link graph: pools identical, and the same distance evaluations."""
    z = load(name)
    g = dict(np.load(os.path.join(HERE, f"ref_pool_search_{name}.npz")))
    p = oracle_py.params(**P, tau=float(z["tau"]))
    oi, od, oc, cc = oracle.pool_search(z["X"], p, z["pool_ids"], z["pool_d"], z["pool_cnt"], z["link_nsg_ids"],
                                        z["link_nsg_deg"], loop)
    assert np.array_equal(oc, g[f"loop{loop}_cnt"])
    assert np.array_equal(oi, g[f"loop{loop}_ids"])
    if name == "c2":
        assert np.array_equal(od, g[f"loop{loop}_d"])
    n = z["X"].shape[0]
    assert cc / (n * (n - 1) / 2) == pytest.approx(float(g[f"loop{loop}_scan"]), rel=1e-5)


PL = dict(K=500, L=500, S=12, R=100, iterations=6, search_L=80, nsg_R=50, search_K=500, controls=20, massq_S=10,
          angle=60.0)


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_prune_link_large(oracle, name):
    """nsg_R = 50, search_K = 500 on the exact 500-NN of 2,000 rows (golden
    ref_prune_large_*.npz): the oracle's edge lists equal the reference's."""
    z = dict(np.load(os.path.join(HERE, f"ref_prune_large_{name}.npz")))
    X = z["X"].astype(np.float32)
    n = X.shape[0]
    pid, pd = oracle.knn(X, np.arange(n, dtype=np.uint32), 500)
    pc = np.full(n, 500, np.uint32)
    p = oracle_py.params(**PL, tau=float(z["tau"]))
    for kind, tag in KINDS:
        gi, _, deg = oracle.prune(kind, X, p, pid, pd, pc, 64)
        assert np.array_equal(deg, z[f"prune_{tag}_deg"].astype(np.uint32)), tag
        for i in range(n):
            assert np.array_equal(gi[i, : deg[i]], z[f"prune_{tag}_ids"][i, : deg[i]].astype(np.uint32)), (tag, i)
        gi, _, deg = oracle.link(kind, X, p, pid, pd, pc, 128)
        assert np.array_equal(deg, z[f"link_{tag}_deg"].astype(np.uint32)), tag
        for i in range(n):
            assert set(gi[i, : deg[i]].tolist()) == set(z[f"link_{tag}_ids"][i, : deg[i]].tolist()), (tag, i)
