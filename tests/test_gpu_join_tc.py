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
    # float rows: not BF16-exact, so the join screens on rounded rows (mode 2)
    index.upload(synth.base("c1", 4000))
    st = index.nndescent(kcna.params(screen=1, **kw))
    assert st["gram_tc"] == 2 and st["bf16_rows"] == 0
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
    assert st1["prune_tc"] == 1 and st0["prune_tc"] == 0
    # the P2K join on Gram tiles evaluates the same pairs as the FP32 one
    assert st0["bridge_comps"] == st1["bridge_comps"] and st0["n_comps"] == st1["n_comps"]


@pytest.mark.parametrize("name,d", [("c3", 96), ("c1", 32)])
def test_screen_join_pools_identical_to_fp32_join(index, monkeypatch, name, d):
    """Float rows (not exact in BF16): the join screens on Gram tiles of the
    rows rounded to BF16 with a bound on the rounding error, and every emitted
    pair is recomputed in FP32, so the pools equal the FP32 join's."""
    _roomy(monkeypatch)
    X = synth.base(name, 12000)
    assert X.shape[1] == d
    kw = dict(K=64, L=64, S=10, R=64, iterations=5, controls=50, recall=1.0, delta=0.0)
    fp32 = _nnd(index, X, 0, **kw)
    scr = _nnd(index, X, 1, **kw)
    assert scr[0]["gram_tc"] == 2 and scr[0]["bf16_rows"] == 0
    assert scr[0]["rescored_pairs"] > 0 and scr[0]["screened_pairs"] == scr[0]["n_comps"]
    for st in (fp32[0], scr[0]):
        _no_overflow(st)
    _same_pools(fp32, scr)


def test_screen_build_matches_fp32_build_c3(index, monkeypatch):
    _roomy(monkeypatch)
    X = synth.base("c3", 15000)
    kw = dict(K=100, L=100, S=10, R=100, iterations=5, search_L=40, nsg_R=40, search_K=100, controls=50,
              recall=1.0, delta=0.0)
    index.upload(X)
    st0 = index.build("nsg", kcna.params(screen=0, **kw))
    g0, deg0, ep0 = index.graph()
    st1 = index.build("nsg", kcna.params(screen=1, **kw))
    g1, deg1, ep1 = index.graph()
    assert st1["gram_tc"] == 2
    assert ep0 == ep1 and np.array_equal(deg0, deg1)
    assert rows_equal_as_sets(g0, deg0, g1, deg1) == 0


def test_screening_error_against_fp64(capsys):
    """The screening bound holds on C3 rows against FP64 distances: Gram
    distances of the BF16-rounded rows (tcgen05, FP32 accumulation) stay below
    (sqrt(d (1 + 2^-15)) + 2^-7 (|x~_i| + |x~_j|))^2 + 2^-14 (|x~_i|^2 + |x~_j|^2)
    for every pair, and the typical relative error is reported."""
    import torch

    from test_gpu_tc import gemm

    X = synth.base("c3", 2048).astype(np.float64)
    Xb = torch.from_numpy(X.astype(np.float32)).to(torch.bfloat16)
    xr = Xb.double().numpy()
    nr = (xr * xr).sum(1)
    G = gemm(Xb.cuda(), Xb.cuda(), M=2048, N=2048, K=X.shape[1]).double().cpu().numpy()
    ds = (nr[:, None] + nr[None, :]).astype(np.float32).astype(np.float64) - 2 * G
    d64 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    a = np.sqrt(nr)
    bound = (np.sqrt(d64 * (1 + 2.0**-15)) + 2.0**-7 * (a[:, None] + a[None, :])) ** 2 + 2.0**-14 * (nr[:, None] + nr[None, :])
    assert (ds <= bound).all()
    off = ~np.eye(2048, dtype=bool)
    rel = np.abs(ds - d64)[off] / np.maximum(d64[off], 1e-12)
    with capsys.disabled():
        print(f"\nC3 BF16 screening error vs FP64: median {np.median(rel):.2e}, 99.9% {np.quantile(rel, 0.999):.2e}, "
              f"max {rel.max():.2e} (relative, off-diagonal)")
