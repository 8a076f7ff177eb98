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


def _pool_diff(gi, gd, gc, ri, rd, rc, rtol):
    """Nodes whose pools differ, comparing each node's ids and their distances
    (within rtol) as sets, and - in a full pool - excusing which of the entries
    tied at its last distance are kept (the reference keeps the one inserted
    last, the GPU the lowest id).  Returns the differing node indices."""
    bad = []
    for i in range(gi.shape[0]):
        c = int(gc[i])
        if c != int(rc[i]):
            bad.append(i)
            continue
        A = dict(zip(gi[i, :c].tolist(), gd[i, :c].tolist()))
        B = dict(zip(ri[i, :c].tolist(), rd[i, :c].tolist()))
        if set(A) == set(B) and all(abs(A[k] - B[k]) <= rtol * abs(B[k]) for k in B):
            continue
        last = max(B.values()) if B else 0.0
        tol = rtol * abs(last)
        A2 = {k for k, v in A.items() if v < last - tol}
        B2 = {k for k, v in B.items() if v < last - tol}
        if A2 == B2 and abs(max(A.values()) - last) <= tol:
            continue
        bad.append(i)
    return bad


def _canonical_dists(X, ids, cnt):
    """Pool distances recomputed by the oracle's canonical FP32 chain (the one
    every GPU kernel uses), so that the GPU's duplicate test - equal distance
    and id - recognises the pools' own entries when a join proposes them."""
    import oracle_py

    O = oracle_py.Oracle()
    out = np.full(ids.shape, np.inf, np.float32)
    for i in range(ids.shape[0]):
        for j in range(int(cnt[i])):
            out[i, j] = O.l2(X[i], X[ids[i, j]])
    return out


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("screen", [0, 1])
def test_gpu_refine_vs_reference(index, name, screen):
    """Two P2K refinement steps (UpdateNhoods + BridgeView, loops 1 and 2) from
    the reference's pools and NSG link graph against the reference's own
    (golden ref_refine_*.npz): the isnew flags of the edges are identical; the
    pools and the join's distance evaluations are identical up to what the two
    implementations cannot share:
      * C1 (float rows): the reference sums distances in AVX lane order, the
        GPU in one FMA chain, so the same pair differs by an ulp; the GPU gets
        the input pools with its own distances (else its duplicate test would
        miss the pools' entries), and distances compare within 1e-6;
      * C2 (integer rows, every distance exact): the reference orders equal
        distances by insertion and the GPU by id; which entry of a tie is
        pushed to a neighbour, or kept at a full pool's end, then differs.
        About 2 % of these 1,000 pools hold a tie; at most 2 % of the nodes
        may differ and the evaluations may differ by 2 %.
    screen = 1 runs the BF16 mode (Gram-tile P2K on the integer C2 rows)."""
    z = load(name)
    r = dict(np.load(os.path.join(HERE, f"ref_refine_{name}.npz")))
    p = kcna.params(**P, tau=float(z["tau"]), step=8, screen=screen)
    n = z["X"].shape[0]
    rtol, max_bad, ctol = (1e-6, 0, 0.005) if name == "c1" else (0.0, n // 50, 0.02)
    pd = _canonical_dists(z["X"], z["pool_ids"], z["pool_cnt"]) if name == "c1" else z["pool_d"]
    index.upload(z["X"])
    index.set_pools(z["pool_ids"], pd, z["pool_cnt"], p)
    index.set_graph(z["link_nsg_ids"], z["link_nsg_deg"], 0)
    comps1 = index.refine(1, p)
    deg1 = z["link_nsg_deg"]
    isnew = index.edge_isnew()
    for i in range(isnew.shape[0]):
        assert isnew[i, : deg1[i]].all()  # loop 1: every edge new
    gi, gd, gc = index.pools()
    W = r["loop1_ids"].shape[1]
    bad = _pool_diff(gi[:, :W], gd[:, :W], gc, r["loop1_ids"], r["loop1_d"], r["loop1_cnt"], rtol)
    assert len(bad) <= max_bad, (len(bad), bad[:10])
    c1 = int(r["loop1_comps"])
    assert abs(comps1 - c1) <= ctol * c1 + 2, (comps1, c1)
    index.set_graph(r["g2_ids"], r["g2_deg"], 0)
    comps2 = index.refine(2, p)
    isnew = index.edge_isnew()
    for i in range(isnew.shape[0]):
        d = int(r["g2_deg"][i])
        assert np.array_equal(isnew[i, :d], r["loop2_isnew"][i, :d]), i
    gi, gd, gc = index.pools()
    bad = _pool_diff(gi[:, :W], gd[:, :W], gc, r["loop2_ids"], r["loop2_d"], r["loop2_cnt"], rtol)
    assert len(bad) <= max_bad, (len(bad), bad[:10])
    c2 = int(r["loop2_comps"])
    assert abs(comps2 - c2) <= ctol * c2 + 2, (comps2, c2)


PL = dict(K=500, L=500, S=12, R=100, iterations=6, search_L=80, nsg_R=50, search_K=500, controls=20, massq_S=10,
          angle=60.0)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("screen", [0, 1])
def test_gpu_prune_link_large_vs_reference(index, name, screen):
    """sync_prune and Link at the C2 flags' sizes (nsg_R = 50, search_K = 500)
    on 500-entry pools, the exact 500-NN of 2,000 rows: the GPU's edge lists
    equal the reference's own (golden ref_prune_large_*.npz).  screen = 1
    selects the BF16 mode (on C2's integer rows: the Gram-tile prune)."""
    z = dict(np.load(os.path.join(HERE, f"ref_prune_large_{name}.npz")))
    X = z["X"].astype(np.float32)
    p = kcna.params(**PL, tau=float(z["tau"]), screen=screen)
    index.upload(X)
    n = X.shape[0]
    pid, pd = index.knn_exact(np.arange(n, dtype=np.uint32), 500)
    pc = np.full(n, 500, np.uint32)
    for kind, tag in KINDS:
        index.set_pools(pid, pd, pc, p)
        index.prune(kind, p)
        g, deg, _ = index.graph()
        ref_deg = z[f"prune_{tag}_deg"].astype(np.uint32)
        ref_ids = z[f"prune_{tag}_ids"].astype(np.uint32)
        assert np.array_equal(deg, ref_deg), (kind, screen)
        for i in range(n):
            assert np.array_equal(g[i, : deg[i]], ref_ids[i, : deg[i]]), (kind, screen, i)
        index.set_pools(pid, pd, pc, p)
        index.link(kind, p)
        g, deg, _ = index.graph()
        ref_deg = z[f"link_{tag}_deg"].astype(np.uint32)
        ref_ids = z[f"link_{tag}_ids"].astype(np.uint32)
        assert np.array_equal(deg, ref_deg), (kind, screen)
        for i in range(n):
            assert set(g[i, : deg[i]].tolist()) == set(ref_ids[i, : deg[i]].tolist()), (kind, screen, i)
