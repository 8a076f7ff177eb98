"""Soundness of the two occlusion screens the tile prunes use, checked on the
CPU against the exact FP32 decisions they replace (numpy float32 emulation of
the kernels' arithmetic; the GPU tests pin the kernels themselves).

* alpha-PG on Gram-exact tiles: a pair the screen proves occluded
  (d(t,p) >= 1 and d(t,p) < min(c, (2 - 4m) c - 16 - a)) must be occluded by
  the reference's own FP32 angle test (src/kgraph.cpp:3181-3186), on random
  and on near-equilateral integer triangles.
* FP8 E4M3 screened tau-MNG prune: with the rows encoded as the kernel encodes
  them and the Gram products perturbed within the kernel's allowance for the
  tensor cores' accumulation, every pair decided "certainly occluded" or
  "certainly not" must agree with the canonical FP32 distance chain."""
import numpy as np

from fastkcna_gb300 import synth

f32 = np.float32


def _thr(angle):
    # as the reference: float angle / 180 times the double pi, cos in double, stored as float
    return f32(np.cos(np.float64(f32(angle) / f32(180.0)) * 3.14159265358979323846264))


def _fma32(x, y, z):
    return (np.float64(x) * np.float64(y) + np.float64(z)).astype(f32)


def _alpha_exact(td, djk, pd, thr):
    """src/kgraph.cpp:3181-3186 in FP32: djk < pd and cos < thr."""
    with np.errstate(divide="ignore", invalid="ignore"):
        num = ((td + djk).astype(f32) - pd).astype(f32) / f32(2.0)
        cs = (num / np.sqrt((td * djk).astype(f32))).astype(f32)
    return (djk < pd) & (cs < thr)


def _alpha_screen(td, dd, pd, thr):
    aux = f32(4.0 * (0.5 - np.float64(thr) + 1e-5))
    k2 = f32(f32(2.0) - aux)
    m = np.minimum(pd, _fma32(k2, pd, (f32(-16.0) - td).astype(f32)))
    return (dd - m < 0) & (f32(0.5) - dd < 0), (dd - pd < 0)


def test_alpha_angle_screen_is_sound():
    rng = np.random.default_rng(5)
    n = 2_000_000
    c = rng.integers(1, 1 << 23, n).astype(np.float64)
    # a <= c and b < c; half of the triangles within 0.1 % of equilateral, some zero sides
    near = rng.random(n) < 0.5
    a = np.where(near, c - rng.integers(0, np.maximum(c * 1e-3, 2).astype(np.int64)), rng.random(n) * c)
    b = np.where(near, c - 1 - rng.integers(0, np.maximum(c * 1e-3, 2).astype(np.int64)), rng.random(n) * c)
    a, b = np.floor(np.clip(a, 0, c)), np.floor(np.clip(b, 0, c - 1))
    b[rng.random(n) < 0.01] = 0
    a[rng.random(n) < 0.01] = 0
    td, dd, pd = a.astype(f32), b.astype(f32), c.astype(f32)
    for angle in (60.0, 45.0, 30.0):
        thr = _thr(angle)
        proven, rng_part = _alpha_screen(td, dd, pd, thr)
        exact = _alpha_exact(td, dd, pd, thr)
        assert not (proven & ~exact).any()  # a proven pair is occluded
        assert not (proven & ~rng_part).any()  # and satisfies RNG
        if angle == 60.0:
            # the screen decides nearly everything the RNG part admits
            assert (rng_part & ~proven).mean() < 0.02


def _e4m3_codes(v):
    a = np.abs(v)
    e = np.floor(np.log2(np.maximum(a, 2.0**-30)))
    step = 2.0 ** (np.maximum(e, -6) - 3)
    return np.sign(v) * np.minimum(np.round(a / step) * step, 448.0)


def _encode(X):
    """fp8_rows_kernel: s = max|x| / 448, codes of x / s, the decoded row's
    squared norm and the inflated bound on |x - s c|."""
    amax = np.abs(X).max(axis=1)
    s = np.where(amax > 0, (amax / f32(448.0)).astype(f32), f32(1.0)).astype(f32)
    codes = _e4m3_codes((X / s[:, None]).astype(f32).astype(np.float64))
    xv = (s[:, None] * codes.astype(f32)).astype(f32).astype(np.float64)
    nn = (xv * xv).sum(1)
    e = np.sqrt(((X.astype(np.float64) - xv) ** 2).sum(1)) * (1 + 1 / 1024) + np.sqrt(nn) * 2.0**-22
    return s.astype(np.float64), codes, nn, e


def _chain(A, B):
    """Canonical FP32 distance: one FMA chain over the dimensions in order."""
    acc = np.zeros(A.shape[0], f32)
    for k in range(A.shape[1]):
        d = (A[:, k] - B[:, k]).astype(f32)
        acc = (np.float64(d) * np.float64(d) + np.float64(acc)).astype(f32)
    return acc


def test_fp8_prune_screen_is_sound_c4():
    X = synth.base("c4", 3000)
    d = X.shape[1]
    s, codes, nn, e = _encode(X)
    rng = np.random.default_rng(11)
    # (q, t, p) triples: t and p among q's 128 nearest, as on the tile
    G64 = X.astype(np.float64)
    nq = 40
    qs = rng.choice(X.shape[0], nq, replace=False)
    tq, pq, qq = [], [], []
    for q in qs:
        dq = ((G64 - G64[q]) ** 2).sum(1)
        order = np.argsort(dq)[1:129]
        ti = rng.integers(0, 128, 200)
        pi = rng.integers(0, 128, 200)
        tq += list(order[ti])
        pq += list(order[pi])
        qq += [q] * 200
    t, p, q = np.array(tq), np.array(pq), np.array(qq)
    D = _chain(X[t], X[p])                       # the exact decision's distance
    pd = _chain(X[q], X[p])                      # d(q,p) as the pool holds it
    G = (codes[t] * codes[p]).sum(1)
    G = G + rng.uniform(-1, 1, G.shape) * 2.0**-9 * np.sqrt((codes[t] ** 2).sum(1) * (codes[p] ** 2).sum(1))
    g = (d + 2) * 2.0**-24 + 1e-5
    nsum = nn[t] + nn[p]
    Dt = nsum - 2 * s[t] * s[p] * G
    dl = 2.0**-7 * nsum
    E = e[t] + e[p]
    decided = 0
    for tau in (10.0, 2.0, 0.0):
        th = (pd - f32(3.0 * tau)).astype(f32).astype(np.float64)
        thp = np.maximum(th, 0)
        rlo, rhi = np.sqrt(thp / (1 - g)), np.sqrt(thp / (1 + g))
        certain_not = (th <= 0) | (Dt - dl >= (E + rlo) ** 2)
        certain_occ = (rhi - E > 0) & (Dt + dl < (rhi - E) ** 2)
        occluded = D.astype(np.float64) < th
        assert not (certain_occ & ~occluded).any()
        assert not (certain_not & occluded).any()
        assert not (certain_occ & certain_not).any()
        decided += (certain_occ | certain_not).sum()
        if tau == 10.0:
            # most pairs decided even on 3,000 rows, whose neighbours lie far apart (on the 1M-row
            # workload the GPU build recomputes about 1,300 pairs in all)
            assert (certain_occ | certain_not).mean() > 0.5
    assert decided > 0
