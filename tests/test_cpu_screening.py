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
