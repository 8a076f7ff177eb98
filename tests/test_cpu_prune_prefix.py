"""The premise of the incremental prune, on the CPU: a node's kept list is a
function of its first S = max(min(search_K, pool capacity), 2) pool entries
(ids, distances) and of min(count, S) - entries beyond them and counts above
S never change it.  Checked for the NSG, tau-MNG and alpha-PG prunes of the
oracle (the restatement of the reference's sync_prune family) and, where the
reference compiled here, of the reference's own prunes (src/kgraph.cpp:
1809-1851, 2833-2876, 3157-3203) on the same pools; a change inside the
prefix does change kept lists (the check is not vacuous)."""
import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import synth

CAP, SEARCH_K, WIDTH = 64, 40, 24


@pytest.fixture(scope="module")
def pools(oracle):
    X = synth.base("c2", 3000)
    ids, d = oracle.knn(X, np.arange(X.shape[0], dtype=np.uint32), CAP)  # self at rank 0
    cnt = np.full(X.shape[0], CAP, np.uint32)
    rng = np.random.default_rng(3)
    # the tail beyond search_K: other ids at larger distances, shorter counts (all above search_K)
    ids_t, d_t, cnt_t = ids.copy(), d.copy(), cnt.copy()
    n = X.shape[0]
    ids_t[:, SEARCH_K:] = rng.integers(0, n, (n, CAP - SEARCH_K)).astype(np.uint32)
    d_t[:, SEARCH_K:] = np.sort(d[:, SEARCH_K - 1 : SEARCH_K] + rng.random((n, CAP - SEARCH_K)).astype(np.float32)
                                * 1000.0, axis=1)
    cnt_t[::3] = rng.integers(SEARCH_K, CAP + 1, cnt_t[::3].size).astype(np.uint32)
    # a change inside the prefix: entries 3 and 4 swapped with 20 and 21 on every fifth row
    ids_p, d_p = ids.copy(), d.copy()
    for a, b in ((3, 20), (4, 21)):
        ids_p[::5, [a, b]] = ids_p[::5, [b, a]]
    return X, (ids, d, cnt), (ids_t, d_t, cnt_t), (ids_p, d_p, cnt)


def _params(lib):
    return lib.params(K=CAP, L=CAP, search_K=SEARCH_K, nsg_R=WIDTH, tau=10.0, angle=60.0)


def _check(prune, params, X, base, tail, pref):
    for kind in (1, 3, 4):
        a = prune(kind, X, params, *base, WIDTH)
        b = prune(kind, X, params, *tail, WIDTH)
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        c = prune(kind, X, params, *pref, WIDTH)
        assert not np.array_equal(a[0], c[0])


def test_kept_lists_depend_on_the_prefix_only_oracle(oracle, pools):
    X, base, tail, pref = pools
    _check(oracle.prune, _params(oracle_py), X, base, tail, pref)


@pytest.mark.skipif(not oracle_py.Reference.available(), reason="reference not compiled here")
def test_kept_lists_depend_on_the_prefix_only_reference(pools):
    ref = oracle_py.Reference()
    X, base, tail, pref = pools
    _check(ref.prune, _params(oracle_py), X, base, tail, pref)
