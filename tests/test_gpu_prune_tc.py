"""Occlusion prune on tensor-core Gram tiles (Gram-exact rows, BF16 mode):
given the same pools, the kept lists equal the FP32 prune's and the oracle's
(the reference's nsg_sync_prune / taumg / alphapg rules) exactly, for the
three rules, with candidate lists spanning one to four 128-row chunks, range
stops, repeated ids (also across a chunk boundary), duplicate rows (the
alpha-PG angle formula's 0/0) and a layer prefix."""
import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu
KIND_CODE = {"nsg": 1, "taumng": 3, "alphapg": 4}


def _pools(index, X, k, dups=True):
    """Exact k-NN pools (self at rank 0); with dups, some rows repeat an
    entry (positions 5/6 and, across the chunk boundary, 128/129)."""
    index.upload(X)
    ids, d = index.knn_exact(np.arange(X.shape[0], dtype=np.uint32), k)
    ids, d = ids.copy(), d.copy()
    if dups:
        for pos in (5, 128):
            rows = np.arange(pos % 7, X.shape[0], 7)
            ids[rows, pos + 1] = ids[rows, pos]
            d[rows, pos + 1] = d[rows, pos]
    return ids, d, np.full(X.shape[0], k, np.uint32)


def _prune(index, ids, d, cnt, kind, screen, **kw):
    p = kcna.params(screen=screen, **kw)
    index.set_pools(ids, d, cnt, p)
    index.prune(kind, p)
    return index.graph()


@pytest.fixture(scope="module")
def c2_rows():
    return synth.base("c2", 12000)


@pytest.mark.parametrize("kind", ["nsg", "taumng", "alphapg"])
@pytest.mark.parametrize("R,search_K", [(50, 500), (8, 300), (128, 130), (32, 64)])
def test_gram_prune_identical_to_fp32(index, c2_rows, kind, R, search_K):
    ids, d, cnt = _pools(index, c2_rows, 500)
    kw = dict(K=500, L=500, search_K=search_K, nsg_R=R, tau=10.0, angle=60.0)
    g0, deg0, _ = _prune(index, ids, d, cnt, kind, 0, **kw)
    g1, deg1, _ = _prune(index, ids, d, cnt, kind, 1, **kw)
    assert np.array_equal(deg0, deg1)
    assert np.array_equal(g0, g1)
    assert deg1.max() <= R and deg1.min() >= 1
    if R == 8:
        assert (deg1 == R).mean() > 0.5  # the range stop is exercised


@pytest.mark.parametrize("kind", ["nsg", "taumng", "alphapg"])
def test_gram_prune_matches_oracle(index, oracle, c2_rows, kind):
    X = c2_rows[:6000]
    ids, d, cnt = _pools(index, X, 400)
    kw = dict(K=400, L=400, search_K=400, nsg_R=50, tau=10.0, angle=60.0)
    g, deg, _ = _prune(index, ids, d, cnt, kind, 1, **kw)
    p = oracle_py.params(**kw)
    oi, od, odeg = oracle.prune(KIND_CODE[kind], X, p, ids, d, cnt, g.shape[1])
    assert np.array_equal(deg, odeg)
    assert np.array_equal(g, oi)


def test_gram_prune_layer_prefix(index, c2_rows):
    """An HNSW layer over the first 5,000 rows (the pools of a prefix hold
    prefix ids only: set_pools rejects others)."""
    index.upload(c2_rows)
    n = 5000
    index.set_size(n)
    ids, d = index.knn_exact(np.arange(n, dtype=np.uint32), 300)
    cnt = np.full(n, 300, np.uint32)
    assert ids.max() < n
    kw = dict(K=300, L=300, search_K=300, nsg_R=40)
    g0, deg0, _ = _prune(index, ids, d, cnt, "hnsw", 0, **kw)
    g1, deg1, _ = _prune(index, ids, d, cnt, "hnsw", 1, **kw)
    assert g1.shape[0] == n
    assert np.array_equal(deg0, deg1) and np.array_equal(g0, g1)


@pytest.mark.parametrize("angle", [45.0, 60.0, 75.0])
def test_gram_alphapg_duplicate_rows(index, oracle, c2_rows, angle):
    """alpha-PG on rows with exact duplicates (distinct ids, equal vectors).
    Two duplicates t, p are at one distance from the node and at distance 0
    from each other, where the reference's angle formula divides 0 by 0 (NaN:
    not occluded); the tile path must take its exact test there.  Angles up to
    60 degrees run on the tiles, 75 on the FP32 prune in both modes."""
    X = c2_rows[:6000].copy()
    X[1::9] = X[0::9][: len(X[1::9])]  # row 9i+1 repeats row 9i
    ids, d, cnt = _pools(index, X, 400, dups=False)
    kw = dict(K=400, L=400, search_K=400, nsg_R=50, angle=angle)
    g0, deg0, _ = _prune(index, ids, d, cnt, "alphapg", 0, **kw)
    g1, deg1, _ = _prune(index, ids, d, cnt, "alphapg", 1, **kw)
    assert np.array_equal(deg0, deg1) and np.array_equal(g0, g1)
    oi, od, odeg = oracle.prune(KIND_CODE["alphapg"], X, oracle_py.params(**kw), ids, d, cnt, g1.shape[1])
    assert np.array_equal(deg1, odeg) and np.array_equal(g1, oi)
    # duplicates stay side by side in the kept lists (neither occludes the other)
    pairs = 0
    for i in range(6000):
        kept = set(g1[i, : deg1[i]].tolist())
        pairs += sum(1 for j in kept if j % 9 == 0 and j + 1 in kept)
    assert pairs > 0
