"""Incremental prune: within a build, the prune after a pool refinement
re-prunes only the nodes whose first search_K pool entries (ids, distances)
or count changed since the previous prune, and restores every other node's
kept list from that prune.  The kept lists are a function of those entries,
the rows and the parameters, so the graphs must equal those of full prunes
bit for bit: the API sequence prune, link, refine, prune against a full
prune of the same pools, and whole builds (Gram-tile prune in BF16 mode, NSG
and tau-MNG; the FP32 warp prune in plain mode; random initial pools) with
the incremental prune on and off."""
import numpy as np
import pytest

from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu

# The API sequence: 50,000 C2 rows (~200 per cluster) with K = 100,
# NN-descent run to the 0.99 recall stop as the 1M build runs it: the
# refinements then change about a tenth of the pools.  (With K above the cluster size the pools stay far from
# converged, every pool changes in every refinement and nothing is skipped.)
N = 50000
KW = dict(K=100, L=100, S=12, R=100, iterations=12, recall=0.99, search_L=40, nsg_R=32, search_K=100, loop_i=2)


@pytest.fixture
def no_overflow(monkeypatch):
    # candidate and reverse-list buffers large enough that nothing overflows:
    # a full buffer keeps whichever entries arrived first
    monkeypatch.setenv("KCNA_CAND_CAP", "8192")
    monkeypatch.setenv("KCNA_REV_CAP", "1024")
    return monkeypatch


def _build(index, monkeypatch, kind, incremental, **kw):
    monkeypatch.setenv("KCNA_PRUNE_INCREMENTAL", "1" if incremental else "0")
    st = index.build(kind, kcna.params(**kw))
    g, deg, ep = index.graph()
    return st, g, deg, ep


@pytest.mark.parametrize("kind,mode", [("nsg", "bf16"), ("taumng", "bf16"), ("nsg", "fp32")])
def test_incremental_prune_build_identical(index, no_overflow, kind, mode):
    """Uniform integer rows (20,000 x 32, no clusters): NN-descent converges
    and the refinements change a few per cent of the pools.  Builds are
    compared bit for bit where tree_grow attached nothing; its parallel
    attachments reserve slots in arrival order, so where it attached nodes,
    two builds differ in some rows even with the same prune, and the
    incremental build may differ from a full one by no more than two full
    builds differ from each other."""
    rng = np.random.default_rng(7)
    X = rng.integers(0, 64, size=(20000, 32)).astype(np.float32)
    index.upload(X)
    kw = dict(K=64, L=64, S=12, R=100, iterations=12, recall=0.99, search_L=40, nsg_R=32, search_K=64, loop_i=2)
    # random initial pools: the learned seed trains with float atomics, so two
    # learned builds need not start from the same pools
    if mode == "bf16":
        kw["screen"] = 1
    if kind == "taumng":
        kw["tau"] = 2.0
    s0, g0, deg0, ep0 = _build(index, no_overflow, kind, False, **kw)
    s1, g1, deg1, ep1 = _build(index, no_overflow, kind, True, **kw)
    for st in (s0, s1):
        assert sum(st["iter_cand_overflow"][: st["iterations"]]) == 0 and st["rev_overflow"] == 0
        assert st["prune_tc"] == (1 if mode == "bf16" else 0)
    assert s0["prune_skipped"] == 0
    # the prunes after the two refinements found unchanged pools (the first prune of a build never skips)
    assert 0 < s1["prune_skipped"] < 2 * X.shape[0]
    assert s0["loop_recall"] == s1["loop_recall"]
    assert ep0 == ep1 and s0["tree_attached"] == s1["tree_attached"]
    if s0["tree_attached"] == 0:
        assert np.array_equal(deg0, deg1) and np.array_equal(g0, g1)
    else:
        from conftest import rows_equal_as_sets
        s2, g2, deg2, _ = _build(index, no_overflow, kind, False, **kw)
        base = rows_equal_as_sets(g0, deg0, g2, deg2)
        assert rows_equal_as_sets(g0, deg0, g1, deg1) <= 1.5 * base + 0.001 * X.shape[0]


@pytest.mark.parametrize("mode", ["bf16", "fp32"])
def test_incremental_prune_after_refine_equals_full_prune(index, monkeypatch, mode):
    X = synth.base("c2", N)
    index.upload(X)
    kw = dict(screen=1) if mode == "bf16" else {}
    p = kcna.params(**KW, **kw)
    monkeypatch.setenv("KCNA_PRUNE_INCREMENTAL", "1")
    index.nndescent(p)
    index.prune("nsg", p)          # full prune: the snapshot
    index.link("nsg", p)           # its prune finds every pool unchanged
    index.refine(1, p)             # BridgeView changes some pools
    index.prune("nsg", p)          # incremental
    g1, deg1, _ = index.graph()
    index.prune("nsg", p)          # incremental, nothing changed: every row restored
    g2, deg2, _ = index.graph()
    monkeypatch.setenv("KCNA_PRUNE_INCREMENTAL", "0")
    index.prune("nsg", p)          # full prune of the same pools
    g0, deg0, _ = index.graph()
    assert np.array_equal(deg0, deg1) and np.array_equal(g0, g1)
    assert np.array_equal(deg0, deg2) and np.array_equal(g0, g2)
    assert deg0.min() >= 1 and deg0.max() <= KW["nsg_R"]
