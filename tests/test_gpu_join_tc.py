"""Local join on tcgen05 Gram tiles (Gram-exact BF16 mode).

On integer rows with squared norms below 2^23 the tile distance
|x|^2 + |y|^2 - 2<x,y> equals the canonical FMA-chain distance, so NN-descent
with the tensor-core join must leave pools identical (ids and distance bits)
to the FP32 register-tile join, iteration by iteration.  The comparison needs
candidate and reverse-list buffers that never overflow (a full buffer keeps
whichever entries arrived first), which the tests check in the statistics."""
import numpy as np
import pytest

from conftest import rows_equal_as_sets
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu


def _roomy(monkeypatch):
    monkeypatch.setenv("KCNA_CAND_CAP", "8192")
    monkeypatch.setenv("KCNA_REV_CAP", "1024")


def _no_overflow(st):
    assert sum(st["iter_cand_overflow"][: st["iterations"]]) == 0
    assert st["rev_overflow"] == 0


def _nnd(index, X, screen, **kw):
    index.upload(X)
    st = index.nndescent(kcna.params(screen=screen, **kw))
    ids, dists, cnt = index.pools()
    return st, ids, dists, cnt


def _same_pools(a, b):
    st0, i0, d0, c0 = a
    st1, i1, d1, c1 = b
    assert np.array_equal(c0, c1)
    live = np.arange(i0.shape[1])[None, :] < c0[:, None]
    assert np.array_equal(i0[live], i1[live])
    assert np.array_equal(d0.view(np.uint32)[live], d1.view(np.uint32)[live])
    assert st0["iterations"] == st1["iterations"]


def test_nndescent_is_reproducible(index, monkeypatch):
    """Premise of the comparisons below: two FP32 runs give identical pools."""
    _roomy(monkeypatch)
    X = synth.base("c2", 12000)
    kw = dict(K=64, L=64, S=10, R=64, iterations=5, controls=50, recall=1.0, delta=0.0)
    a = _nnd(index, X, 0, **kw)
    b = _nnd(index, X, 0, **kw)
    _no_overflow(a[0])
    _same_pools(a, b)


@pytest.mark.parametrize("d", [128, 96, 32])
def test_tc_join_pools_identical_to_fp32_join(index, monkeypatch, d):
    _roomy(monkeypatch)
    X = np.ascontiguousarray(synth.base("c2", 12000)[:, :d])
    kw = dict(K=64, L=64, S=10, R=64, iterations=5, controls=50, recall=1.0, delta=0.0)
    fp32 = _nnd(index, X, 0, **kw)
    tc = _nnd(index, X, 1, **kw)
    assert fp32[0]["gram_tc"] == 0 and tc[0]["gram_tc"] == 1 and tc[0]["bf16_rows"] == 1
    for st in (fp32[0], tc[0]):
        _no_overflow(st)
    _same_pools(fp32, tc)


def test_tc_join_large_lists(index, monkeypatch):
    """L = 300 with R = 100: old lists beyond 128 rows exercise the rotating
    column slots (chunks 2, 3, ...)."""
    _roomy(monkeypatch)
    X = synth.base("c2", 20000)
    kw = dict(K=300, L=300, S=12, R=100, iterations=4, controls=50, recall=1.0, delta=0.0)
    fp32 = _nnd(index, X, 0, **kw)
    tc = _nnd(index, X, 1, **kw)
    assert tc[0]["gram_tc"] == 1
    for st in (fp32[0], tc[0]):
        _no_overflow(st)
    _same_pools(fp32, tc)


def test_gram_exact_mode_rejects_unsafe_rows(index):
    kw = dict(K=32, L=32, S=8, R=32, iterations=2, controls=20)
    # float rows: not BF16-exact
    index.upload(synth.base("c1", 4000))
    assert index.nndescent(kcna.params(screen=1, **kw))["gram_tc"] == 0
    # integer rows whose squared norm reaches 2^23: BF16 rows yes, Gram tiles no
    X = synth.base("c2", 4000).copy()
    X[7, :] = 256.0
    index.upload(X)
    st = index.nndescent(kcna.params(screen=1, **kw))
    assert st["bf16_rows"] == 1 and st["gram_tc"] == 0
    # d not a multiple of 8
    index.upload(np.ascontiguousarray(synth.base("c2", 4000)[:, :100]))
    st = index.nndescent(kcna.params(screen=1, **kw))
    assert st["bf16_rows"] == 1 and st["gram_tc"] == 0


def test_tc_join_build_matches_fp32_build(index, monkeypatch):
    """Whole FastNSG build: with identical pools the prune, link, P2K (also on
    Gram tiles here) and tree_grow steps see identical inputs, so the graphs
    agree."""
    _roomy(monkeypatch)
    X = synth.base("c2", 15000)
    kw = dict(K=100, L=100, S=10, R=100, iterations=5, search_L=40, nsg_R=32, search_K=100, controls=50,
              recall=1.0, delta=0.0)
    index.upload(X)
    st0 = index.build("nsg", kcna.params(screen=0, **kw))
    g0, deg0, ep0 = index.graph()
    st1 = index.build("nsg", kcna.params(screen=1, **kw))
    g1, deg1, ep1 = index.graph()
    assert st1["gram_tc"] == 1
    assert ep0 == ep1
    assert np.array_equal(deg0, deg1)
    assert rows_equal_as_sets(g0, deg0, g1, deg1) == 0
    assert st0["loop_recall"][-1] == st1["loop_recall"][-1]
    # the P2K join on Gram tiles evaluates the same pairs as the FP32 one
    assert st0["bridge_comps"] == st1["bridge_comps"] and st0["n_comps"] == st1["n_comps"]
