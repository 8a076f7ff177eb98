"""Seeded synthetic datasets with the shapes of the FastKCNA benchmark sets.

The paper's datasets (Sift1M, Deep1M, Gist1M, ...) are not available here, so
each workload is a seeded mixture with the named shape and value range:

* ``c1``: 20,000 + 1,000 x 32 float, 16-component isotropic Gaussian mixture,
  centres U[-1,1]^32, sigma 0.1, equal weights.
* ``c2``: 1,000,000 + 10,000 x 128 float holding integers 0..255: 256 centres
  U[0,160]^128, per-dimension Laplace noise (scale 12), rounded and clipped
  (stands in for Sift1M).
* ``c3``: 1,000,000 + 10,000 x 96, 1,024 centres N(0, I), sigma 0.35, rows
  L2-normalised (stands in for Deep1M).
* ``c4``: 1,000,000 + 1,000 x 960 nonnegative: |GMM| with 512 centres
  |N(0, 0.5)|, sigma 0.2 (stands in for Gist1M).
* ``c5``: as ``c2`` with 2,000,000 base rows.

Seeds: 2024 for base rows (the reference's default seed, src/kgraph.h:21),
2025 for queries, 2026 for mixture centres.  ``n`` may be given to draw a
smaller prefix-independent sample of the same distribution.
"""
from __future__ import annotations

import struct

import numpy as np

SEED_BASE, SEED_QUERY, SEED_CENTRES = 2024, 2025, 2026

SPECS = {
    "c1": dict(n=20_000, q=1_000, d=32),
    "c2": dict(n=1_000_000, q=10_000, d=128),
    "c3": dict(n=1_000_000, q=10_000, d=96),
    "c4": dict(n=1_000_000, q=1_000, d=960),
    "c5": dict(n=2_000_000, q=10_000, d=128),
}


def _centres(name: str) -> np.ndarray:
    rng = np.random.default_rng(SEED_CENTRES)
    d = SPECS[name]["d"]
    if name == "c1":
        return rng.uniform(-1.0, 1.0, size=(16, d))
    if name in ("c2", "c5"):
        return rng.uniform(0.0, 160.0, size=(256, d))
    if name == "c3":
        return rng.standard_normal(size=(1024, d))
    if name == "c4":
        return np.abs(rng.normal(0.0, 0.5, size=(512, d)))
    raise KeyError(name)


def _draw(name: str, n: int, seed: int, chunk: int = 1 << 17, labels: np.ndarray | None = None) -> np.ndarray:
    d = SPECS[name]["d"]
    cen = _centres(name)
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        m = e - s
        lab = rng.integers(0, cen.shape[0], size=m)
        if labels is not None:
            labels[s:e] = lab
        if name == "c1":
            x = cen[lab] + 0.1 * rng.standard_normal(size=(m, d))
        elif name in ("c2", "c5"):
            x = cen[lab] + rng.laplace(0.0, 12.0, size=(m, d))
            x = np.clip(np.rint(x), 0, 255)
        elif name == "c3":
            x = cen[lab] + 0.35 * rng.standard_normal(size=(m, d))
            x /= np.linalg.norm(x, axis=1, keepdims=True)
        else:  # c4
            x = np.abs(cen[lab] + 0.2 * rng.standard_normal(size=(m, d)))
        out[s:e] = x.astype(np.float32)
    return out


def centres(name: str) -> np.ndarray:
    """The mixture centres the rows of a workload are drawn around."""
    return _centres(name).copy()


def base(name: str, n: int | None = None) -> np.ndarray:
    """Base rows (float32, C-contiguous)."""
    return _draw(name, SPECS[name]["n"] if n is None else n, SEED_BASE)


def queries(name: str, q: int | None = None) -> np.ndarray:
    """Query rows drawn from the same mixture with the query seed."""
    return _draw(name, SPECS[name]["q"] if q is None else q, SEED_QUERY)


def base_labels(name: str, n: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Base rows (as base()) and the mixture component each was drawn from."""
    n = SPECS[name]["n"] if n is None else n
    lab = np.empty(n, np.int32)
    return _draw(name, n, SEED_BASE, labels=lab), lab


def query_labels(name: str, q: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Query rows (as queries()) and the mixture component each was drawn from."""
    q = SPECS[name]["q"] if q is None else q
    lab = np.empty(q, np.int32)
    return _draw(name, q, SEED_QUERY, labels=lab), lab


def write_lshkit(path: str, x: np.ndarray) -> None:
    """lshkit file: u32 header {element size 4, rows, cols} then rows
    (the layout read by Matrix::load_lshkit, src/kgraph-data.h:262-274)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    with open(path, "wb") as f:
        f.write(struct.pack("<III", 4, x.shape[0], x.shape[1]))
        f.write(x.tobytes())


def read_lshkit(path: str) -> np.ndarray:
    """Reads an lshkit float file; the row count follows from the file size
    as in Matrix::load (src/kgraph-data.h:161-177)."""
    with open(path, "rb") as f:
        hdr = f.read(12)
        if len(hdr) != 12:
            raise IOError(path)
        esz, _rows, cols = struct.unpack("<III", hdr)
        if esz != 4:
            raise IOError(path)
        raw = np.frombuffer(f.read(), dtype=np.float32)
    n = raw.size // cols
    return raw[: n * cols].reshape(n, cols).copy()
