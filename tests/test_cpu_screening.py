"""Screening representations against FP64, on the CPU: the BF16 rounding the
Gram-tile screen uses (C3) and an FP8 E4M3 encoding with per-vector scales
(C4, the high-dimension form), emulated in numpy.  Each prints the relative
error of the squared distance of the encoded rows and checks the bound the
screen relies on: | |x~ - y~| - |x - y| | <= E(x) + E(y), with E the encoding
error of one row."""
import numpy as np

from fastkcna_gb300 import synth


def _bf16(x):
    """Round-to-nearest-even to BF16, as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _e4m3(v):
    """Round-to-nearest-even to FP8 E4M3 (3 mantissa bits, min normal 2^-6,
    subnormal step 2^-9, max 448), as float64."""
    a = np.abs(v)
    e = np.floor(np.log2(np.maximum(a, 2.0**-30)))
    step = 2.0 ** (np.maximum(e, -6) - 3)
    q = np.round(a / step) * step  # numpy rounds half to even
    return np.sign(v) * np.minimum(q, 448.0)


def _fp8_rows(X):
    s = np.abs(X).max(axis=1, keepdims=True) / 448.0
    s[s == 0] = 1.0
    return _e4m3(X / s) * s, s[:, 0]


def _pair_errors(X, Xq, n=600, seed=0):
    rng = np.random.default_rng(seed)
    i = rng.choice(X.shape[0], n, replace=False)
    A, Aq = X[i], Xq[i]
    d = ((A[:, None, :] - A[None, :, :]) ** 2).sum(-1)
    dq = ((Aq[:, None, :] - Aq[None, :, :]) ** 2).sum(-1)
    off = ~np.eye(n, dtype=bool)
    return i, d, dq, off


def _report(tag, d, dq, off):
    rel = np.abs(dq - d)[off] / np.maximum(d[off], 1e-30)
    print(f"\n{tag} vs FP64: median {np.median(rel):.2e}, 99.9% {np.quantile(rel, 0.999):.2e}, max {rel.max():.2e}")
    return rel


def test_bf16_screening_error_c3(capsys):
    X = synth.base("c3", 4000).astype(np.float64)
    Xq = _bf16(X)
    i, d, dq, off = _pair_errors(X, Xq)
    E = np.sqrt(((Xq - X) ** 2).sum(1))[i]
    assert (np.abs(np.sqrt(dq) - np.sqrt(d)) <= E[:, None] + E[None, :] + 1e-12)[off].all()
    assert (E <= 2.0**-8 * np.sqrt((X[i] ** 2).sum(1)) + 1e-12).all()  # relative rounding 2^-8 per element
    with capsys.disabled():
        rel = _report("C3 BF16 rows, squared distance", d, dq, off)
    assert np.median(rel) < 2e-3


def test_fp8_e4m3_screening_error_c4(capsys):
    X = synth.base("c4", 3000).astype(np.float64)
    assert X.shape[1] == 960
    Xq, s = _fp8_rows(X)
    i, d, dq, off = _pair_errors(X, Xq)
    E = np.sqrt(((Xq - X) ** 2).sum(1))[i]
    assert (np.abs(np.sqrt(dq) - np.sqrt(d)) <= E[:, None] + E[None, :] + 1e-9)[off].all()
    # per-element bound: 2^-4 relative in the normal range, half the subnormal step below it
    nx = np.sqrt((X[i] ** 2).sum(1))
    assert (E <= 2.0**-4 * nx + s[i] * 2.0**-10 * np.sqrt(960) + 1e-9).all()
    with capsys.disabled():
        rel = _report("C4 FP8 E4M3 rows (per-vector scales), squared distance", d, dq, off)
        # the screen's radius inflation: (|x - y| + E(x) + E(y))^2 / |x - y|^2 at the pool scale
        nn = np.sort(d, axis=1)[:, 1:51]
        infl = ((np.sqrt(nn) + 2 * np.median(E)) ** 2 / nn).mean()
        print(f"C4 FP8 bound inflates a 50-NN radius by {100 * (infl - 1):.0f} % on average")
    assert np.median(rel) < 0.1


def _gram_d2(A, B):
    return np.maximum((A * A).sum(1)[:, None] + (B * B).sum(1)[None, :] - 2.0 * A @ B.T, 0.0)


def test_screen_pass_ratio_c4(capsys):
    """How many pairs each screen lets through at a converged pool radius on
    C4: the radius is each row's 4th-NN distance among 8,000 rows (the scale
    of a 500-NN radius among 1M rows); a pair passes the exact test when
    d <= r, a screen when the encoded distance is within its bound.  The
    distances of C4 concentrate (a random pair sits ~9 % beyond the 500-NN
    radius), so the FP8 bound, ~14 % wider, passes several times the exact
    pairs and every one of them would need an FP32 recompute."""
    X = synth.base("c4", 8000).astype(np.float64)
    Xq, _ = _fp8_rows(X)
    Xb = _bf16(X)
    E8 = np.sqrt(((Xq - X) ** 2).sum(1))
    Eb = np.sqrt(((Xb - X) ** 2).sum(1))
    nq = (Xq * Xq).sum(1)
    i = np.arange(200)
    d = _gram_d2(X[i], X)
    r = np.sort(d, axis=1)[:, 4][:, None]
    exact = int((d <= r).sum())
    b8 = (np.sqrt(r) + E8[i, None] + E8[None, :]) ** 2 + 2.0**-8 * (nq[i, None] + nq[None, :])
    p8 = int((_gram_d2(Xq[i], Xq) <= b8).sum())
    bb = (np.sqrt(r) + Eb[i, None] + Eb[None, :]) ** 2
    pb = int((_gram_d2(Xb[i], Xb) <= bb).sum())
    with capsys.disabled():
        print(f"\nC4 pairs passing at a 500-NN-scale radius: exact {exact}, FP8 E4M3 screen {p8} "
              f"({p8 / exact:.1f}x), BF16 screen {pb} ({pb / exact:.2f}x)")
    assert p8 >= pb >= exact  # every screen is a superset of the exact test
    assert p8 > 2 * exact and pb < 1.6 * exact
