"""The workload shapes beyond the headline build: C4's high dimension
(d = 960, FastTauMNG, tau = 10) on the FP32 kernels, with the prune checked
bit for bit against the oracle on the GPU's own pools (the FP8-screened prune
of the same rows is pinned in test_gpu_prune_fp8.py), and C5's size (2M x
128 integer rows, FastAlphaPG, learned seed + BF16, the alpha-PG prune on Gram
tiles) against the plain FP32 build of the same rows."""
import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu


def _exact_recall(index, ids, cnt, k, sample):
    ti, _ = index.knn_exact(sample, k + 1)
    hit = 0
    for r, q in enumerate(sample):
        truth = set(ti[r].tolist()) - {int(q)}
        got = set(ids[q, : min(cnt[q], k + 1)].tolist()) - {int(q)}
        hit += len(truth & got) / len(truth)
    return hit / len(sample)


def test_c4_high_dimension_taumng(index, oracle):
    X = synth.base("c4", 6000)
    assert X.shape[1] == 960
    kw = dict(K=100, L=100, S=12, R=100, iterations=6, search_L=80, nsg_R=50, search_K=100, tau=10.0,
              controls=50, recall=0.99)
    index.upload(X)
    st = index.nndescent(kcna.params(**kw))
    pid, pd, pc = index.pools()
    rng = np.random.default_rng(3)
    sample = rng.choice(X.shape[0], 200, replace=False).astype(np.uint32)
    # NN-descent is stochastic: the GPU pools' exact recall@100 against the
    # oracle restatement's on the same rows (the reference compiled from its
    # sources reaches 0.944 here, the oracle 0.945)
    opid, _, opc, _ = oracle.nndescent(X, oracle_py.params(**kw), nthreads=8)
    gpu_rec = _exact_recall(index, pid, pc, 100, sample)
    orc_rec = _exact_recall(index, opid, opc, 100, sample)
    assert abs(gpu_rec - orc_rec) <= 0.01, (gpu_rec, orc_rec)
    # prune of the GPU's pools, against the oracle's prune of the same pools
    p = kcna.params(**kw)
    index.set_pools(pid, pd, pc, p)
    index.prune("taumng", p)
    g, deg, _ = index.graph()
    oi, od, odeg = oracle.prune(3, X, oracle_py.params(**kw), pid, pd, pc, g.shape[1])
    assert np.array_equal(deg, odeg)
    assert np.array_equal(g, oi)
    assert st["gram_tc"] == 0  # d > 128: FP32 kernels throughout


def test_c5_two_million_alphapg_learned_bf16():
    X = synth.base("c5")
    assert X.shape == (2_000_000, 128)
    kw = dict(K=500, L=500, S=12, R=100, iterations=12, search_L=80, nsg_R=50, search_K=500, massq_S=10,
              loop_i=2, step=10, angle=60.0, recall=0.99)
    with kcna.Index(0) as ix:
        ix.upload(X)
        st = ix.build("alphapg", kcna.params(learned_seed=1, screen=1, **kw))
        g1, d1, _ = ix.graph()
        st0 = ix.build("alphapg", kcna.params(**kw))
        g0, d0, _ = ix.graph()
    assert st["gram_tc"] == 1 and st["prune_tc"] == 1  # alpha-PG (angle 60) prunes on the Gram tiles
    assert st["loop_recall"][-1] >= 0.99 and st0["loop_recall"][-1] >= 0.99
    assert st["iterations"] < st0["iterations"]  # the learned seed cuts NN-descent iterations
    assert d1.max() <= 50 and d0.max() <= 50
    assert abs(float(d1.mean()) - float(d0.mean())) < 0.5
    assert st["phase_ms"]["prune"] < st0["phase_ms"]["prune"]
    print(f"\nC5 2M alpha-PG: learned+BF16 {st['total_time']:.2f} s ({st['iterations']} iterations), "
          f"plain FP32 {st0['total_time']:.2f} s ({st0['iterations']} iterations)")


def test_c2_exact_knn_10k_subset_bit_exact():
    """C2 at full size (1,000,000 x 128 integer rows): the exact 100-NN of a
    seeded 10,000-row subset from the library's distance kernel equals, ids and
    distances bit for bit, an independent FP64 computation in torch on the same
    GPU (|x|^2 + |y|^2 - 2<x, y> is an integer below 2^24 here, so FP64 and the
    canonical FP32 chain are both exact) with ties broken by the lower id, as
    the reference's LinearSearch does (src/kgraph.cpp:309-330)."""
    import torch

    X = synth.base("c2")
    n = X.shape[0]
    sub = np.random.default_rng(2024).choice(n, 10_000, replace=False).astype(np.uint32)
    k = 100
    with kcna.Index(0) as ix:
        ix.upload(X)
        gi, gd = ix.knn_exact(sub, k)
    dev = torch.device("cuda", 0)
    Xd = torch.from_numpy(X).to(dev, torch.float64)
    xn = (Xd * Xd).sum(1)
    ids_all = torch.arange(n, device=dev, dtype=torch.int64)
    for s in range(0, sub.size, 500):
        q = torch.from_numpy(sub[s: s + 500].astype(np.int64)).to(dev)
        d = xn[q][:, None] + xn[None, :] - 2.0 * (Xd[q] @ Xd.T)
        d[torch.arange(q.numel(), device=dev), q] = 2.0 ** 40  # the row itself is not its neighbour
        key = d.to(torch.int64) * (1 << 21) + ids_all  # exact integers below 2^24: (distance, id) in one key
        top = torch.topk(key, k, dim=1, largest=False, sorted=True).values
        ti = (top % (1 << 21)).cpu().numpy().astype(np.uint32)
        td = (top // (1 << 21)).cpu().numpy().astype(np.float32)
        assert np.array_equal(gi[s: s + 500], ti), s
        assert np.array_equal(gd[s: s + 500], td), s
