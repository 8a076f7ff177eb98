"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Bit-exact where the path is deterministic (exact k-NN, prune, link, beam
search); recall-based where the reference itself is stochastic (NN-descent,
P2K refinement, full builds).
"""
import numpy as np
import pytest

import oracle_py
from conftest import recall_at, rows_equal_as_sets
from fastkcna_gb300 import synth

pytestmark = pytest.mark.gpu

KINDS = {1: "nsg", 3: "taumng", 4: "alphapg"}


@pytest.fixture(scope="module")
def c1():
    return synth.base("c1", 6000)


@pytest.fixture(scope="module")
def c2():
    return synth.base("c2", 6000)


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_knn_exact_bit_identical(index, oracle, name, c1, c2):
    X = c1 if name == "c1" else c2
    index.upload(X)
    ids = np.arange(0, X.shape[0], 37, dtype=np.uint32)
    gi, gd = index.knn_exact(ids, 100)
    oi, od = oracle.knn(X, ids, 100)
    assert np.array_equal(gd, od)
    assert np.array_equal(gi, oi)


def test_knn_edge_sizes(index, oracle):
    X = synth.base("c1", 257)  # ragged n, d=32
    index.upload(X)
    ids = np.array([0, 1, 255, 256], np.uint32)
    gi, gd = index.knn_exact(ids, 256)  # k = n - 1: every other row
    oi, od = oracle.knn(X, ids, 256)
    assert np.array_equal(gi, oi) and np.array_equal(gd, od)


def test_knn_queries(index, oracle, c2):
    index.upload(c2)
    Q = synth.queries("c2", 50)
    gi, gd = index.knn_queries(Q, 10)
    oi, od = oracle.knn_queries(c2, Q, 10)
    assert np.array_equal(gi, oi) and np.array_equal(gd, od)


def test_knn_duplicate_rows_tie_break(index, oracle):
    X = synth.base("c2", 500)
    X[100:200] = X[0]  # many exact ties
    index.upload(X)
    ids = np.array([0, 5, 150], np.uint32)
    gi, gd = index.knn_exact(ids, 120)
    oi, od = oracle.knn(X, ids, 120)
    assert np.array_equal(gi, oi) and np.array_equal(gd, od)


def _pools(oracle, X, **kw):
    p = oracle_py.params(**kw)
    pid, pd, pc, st = oracle.nndescent(X, p, nthreads=1)
    return p, pid, pd, pc


@pytest.mark.parametrize("kind", [1, 3, 4])
@pytest.mark.parametrize("name", ["c1", "c2"])
def test_prune_bit_identical(index, oracle, kind, name, c1, c2):
    from fastkcna_gb300 import kcna

    X = c1 if name == "c1" else c2
    tau = 0.05 if name == "c1" else 10.0
    kw = dict(K=100, L=100, S=10, R=100, iterations=4, search_L=40, nsg_R=32, search_K=100, tau=tau, angle=60.0)
    p, pid, pd, pc = _pools(oracle, X, **kw)
    index.upload(X)
    kp = kcna.params(**kw)
    index.set_pools(pid, pd, pc, kp)
    index.prune(KINDS[kind], kp)
    g, deg, _ = index.graph()
    oi, od, odeg = oracle.prune(kind, X, p, pid, pd, pc, g.shape[1])
    assert np.array_equal(deg, odeg)
    assert np.array_equal(g, oi)


@pytest.mark.parametrize("kind", [1, 3, 4])
def test_link_bit_identical(index, oracle, kind, c1):
    from fastkcna_gb300 import kcna

    kw = dict(K=100, L=100, S=10, R=100, iterations=4, search_L=40, nsg_R=16, search_K=100, tau=0.05, angle=60.0)
    p, pid, pd, pc = _pools(oracle, c1, **kw)
    index.upload(c1)
    kp = kcna.params(**kw)
    index.set_pools(pid, pd, pc, kp)
    index.link(KINDS[kind], kp)
    g, deg, _ = index.graph()
    oi, od, odeg = oracle.link(kind, c1, p, pid, pd, pc, g.shape[1])
    assert np.array_equal(deg, odeg)
    assert rows_equal_as_sets(g, deg, oi, odeg) == 0
    assert np.array_equal(g, oi)


def test_beam_search_bit_identical(index, oracle, c1):
    kw = dict(K=100, L=100, S=10, R=100, iterations=4, search_L=40, nsg_R=24, search_K=100)
    p, pid, pd, pc = _pools(oracle, c1, **kw)
    W = 64
    gi, gd, gdeg = oracle.link(1, c1, p, pid, pd, pc, W)
    index.upload(c1)
    index.set_graph(gi, gdeg, 0)
    Q = synth.queries("c1", 200)
    rng = np.random.default_rng(7)
    L = 40
    init = np.stack([rng.choice(c1.shape[0], L, replace=False) for _ in range(Q.shape[0])]).astype(np.uint32)
    ki, kd = index.search(Q, L, 10, init)
    oi, od = oracle.beam_search(c1, gi, gdeg, Q, init, L, 10)
    assert np.array_equal(ki, oi) and np.array_equal(kd, od)


def test_nndescent_recall_matches_oracle(index, oracle):
    X = synth.base("c1", 20000)
    kw = dict(K=100, L=100, S=10, R=100, iterations=6, search_L=40, nsg_R=32, search_K=100, controls=100)
    index.upload(X)
    st = index.nndescent(**kw)
    _, _, _, ost = oracle.nndescent(X, oracle_py.params(**kw), nthreads=8)
    g = st["loop_recall"][0]
    o = ost.loop_recall[0]
    # stochastic path: control recall on the same control nodes.  On these rows
    # (20k x 32 floats, K = L = 100) the batched joins trail the reference's
    # locked inserts after five iterations: GPU 0.984, oracle 0.986, the
    # reference compiled from its sources 0.986-0.987 (larger candidate and
    # reverse buffers, or crediting found joiners at other insert positions,
    # leave 0.983-0.984); on the C2 workload the GPU is within 0.002 of the
    # reference's own builds (tests/test_gpu_quality.py).  Bar here: 0.004.
    assert abs(g - o) <= 0.004, (g, o, st)
    # exact recall on a subset, independent of the control estimator
    pid, pd, pc = index.pools()
    ids = np.arange(0, X.shape[0], 200, dtype=np.uint32)
    ti, _ = oracle.knn(X, ids, 100)
    r = recall_at(pid[ids], ti, 100)
    assert r >= o - 0.02, (r, o)
    # pools sorted, no duplicate ids, no self
    for i in ids:
        row = pid[i, : pc[i]]
        assert len(set(row.tolist())) == len(row) and i not in row
        assert np.all(np.diff(pd[i, : pc[i]]) >= 0)


def _cluster_starts(X, Q, ep, L, name="c1"):
    """Start nodes per query: the entry point and L - 1 seeded random rows of
    the query's own cluster (nearest mixture centre)."""
    cen = synth.centres(name).astype(np.float32)
    lab_x = np.argmin(((X[:, None, :] - cen[None]) ** 2).sum(-1), axis=1)
    lab_q = np.argmin(((Q[:, None, :] - cen[None]) ** 2).sum(-1), axis=1)
    members = [np.flatnonzero(lab_x == c) for c in range(cen.shape[0])]
    out = np.empty((Q.shape[0], L), np.uint32)
    for qi in range(Q.shape[0]):
        out[qi, 0] = ep
        out[qi, 1:] = np.random.default_rng(qi).choice(members[lab_q[qi]], size=L - 1, replace=False)
    return out


@pytest.mark.parametrize("kind", ["nsg", "taumng", "alphapg"])
def test_build_search_recall(index, oracle, kind):
    """Search recall@10 of the GPU build against the oracle build of the same
    rows and flags, both graphs searched by the same GPU searcher.  C1's 16
    clusters hold 1,250 rows each against K = 100, so the graph is one island
    per cluster joined only by tree_grow's links, and a search from the entry
    point and random nodes reaches a query's cluster by chance: whole clusters
    are found or missed per build (measured on both builders: recall 0.93 or
    0.999 by seed).  Beams started inside the query's cluster measure the
    graph itself; there the two builders agree to 0.0005 over three seeds at
    L = 12 and 16 (recall 0.87-0.92), and the bar is 0.002."""
    X = synth.base("c1", 20000)
    Q = synth.queries("c1", 2000)
    kw = dict(K=100, L=100, S=10, R=100, iterations=6, search_L=40, nsg_R=32, search_K=100, massq_S=10,
              angle=60.0, tau=0.05, loop_i=2)
    index.upload(X)
    st = index.build(kind, **kw)
    g, deg, ep = index.graph()
    n = X.shape[0]
    assert deg.max() <= 32 + 1 and np.all(g[np.arange(g.shape[1])[None, :] < deg[:, None]] < n)
    # connectivity from the entry point (tree_grow)
    seen = np.zeros(n, bool)
    seen[ep] = True
    front = [ep]
    while front:
        nxt = []
        for u in front:
            for v in g[u, : deg[u]]:
                if not seen[v]:
                    seen[v] = True
                    nxt.append(v)
        front = nxt
    assert seen.all()
    truth, _ = oracle.knn_queries(X, Q, 10)
    r_gpu = {L: recall_at(index.search(Q, L, 10, init_ids=_cluster_starts(X, Q, ep, L))[0], truth, 10)
             for L in (12, 16)}
    # the oracle build of the same kind, searched by the same GPU searcher
    kid = {"nsg": 1, "taumng": 3, "alphapg": 4}[kind]
    og, odeg, ost = oracle.build(kid, X, oracle_py.params(**kw), width=g.shape[1], nthreads=8)
    index.set_graph(og, odeg, ost.ep)
    r_orc = {L: recall_at(index.search(Q, L, 10, init_ids=_cluster_starts(X, Q, ost.ep, L))[0], truth, 10)
             for L in (12, 16)}
    for L in (12, 16):
        assert abs(r_gpu[L] - r_orc[L]) <= 0.002, (L, r_gpu, r_orc, st)
