"""Generates tests/golden/ref_quality_c2.npz: build quality of the reference's
own FastNSG builds on subsets of the C2 workload, the bar the GPU build is held
to (recall@K and search recall@10 within 0.002 of the reference CPU build).

The reference (oracle/_ref/libkcna_ref.so, compiled unmodified from its
sources by oracle/build_ref.sh) builds the first n rows of the seeded C2
generator (integer-valued 256-cluster mixture, d = 128) with the C2 flags
(-K 500 -L 500 -S 12 -R 100 --search_L 80 --nsg_R 50 --search_K 500
--massq_S 10 --loop_i 2 --step 10) and the bench's stop rule (-I 12
--recall 0.99), through its public API (KGraph::create + buildFastNSG,
src/kgraph.cpp:3796-3851), twice per size (OpenMP timing makes its builds
differ slightly).  Recorded per build:
  * the run CSV's recall row: control recall@K after every NN-descent
    iteration, again after NN-descent, then after every BridgeView loop
    (src/kgraph.cpp:1397, 3801-3802, 3842-3843).  The reference's 100
    control nodes (GenerateControl, :363-387) are the ones the GPU library
    uses, so both are scored on the same nodes;
  * search recall@10 of the built NSG over 10,000 C2 queries with the
    reference's own beam search (get_neighbors, :1560-1623), beam L from the
    entry point plus L - 1 seeded random nodes, for L in BEAMS.
Sizes: 100,000 rows, where the reference's NN-descent stalls near recall 0.80
(few nodes keep finding new neighbours) - a regime sensitive to the join's
semantics - and 200,000 rows, where it converges past 0.99.

Usage: python tests/golden/make_golden_quality.py   (needs oracle/_ref built
here; about five minutes on 8 cores)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    sys.path.insert(0, p)

import oracle_py  # noqa: E402
from fastkcna_gb300 import synth  # noqa: E402

SIZES = (100_000, 200_000)
BUILDS = 2
NQ = 10_000
BEAMS = (10, 20, 40, 80)
FLAGS = dict(K=500, L=500, S=12, R=100, iterations=12, search_L=80, nsg_R=50, search_K=500, massq_S=10,
             loop_i=2, step=10, angle=60.0, recall=0.99, controls=100, seed=2024)


def exact10(X, Q):
    """Exact 10-NN, ties by the lower id (float64 norm expansion; the rows are
    integers, so every distance is exact)."""
    X64 = X.astype(np.float64)
    xn = (X64 * X64).sum(1)
    out = np.empty((Q.shape[0], 10), np.int64)
    for s in range(0, Q.shape[0], 512):
        q = Q[s: s + 512].astype(np.float64)
        d = xn[None, :] + (q * q).sum(1)[:, None] - 2.0 * (q @ X64.T)
        part = np.argpartition(d, 10, axis=1)[:, :11]
        for i in range(q.shape[0]):
            c = part[i]
            out[s + i] = c[np.lexsort((c, d[i, c]))[:10]]
    return out


def start_nodes(n, ep, L):
    """The entry point plus L - 1 seeded random nodes (the same for every query)."""
    rng = np.random.default_rng(7)
    extra = rng.choice(n, size=L, replace=False)
    return np.concatenate([[ep], extra[extra != ep][: L - 1]]).astype(np.uint32)


def main():
    ref = oracle_py.Reference()
    threads = os.cpu_count() or 1
    out = {"beams": np.asarray(BEAMS, np.int32), "sizes": np.asarray(SIZES, np.int64),
           "builds": np.int32(BUILDS), "nq": np.int32(NQ)}
    Q = synth.queries("c2", NQ)
    for n in SIZES:
        X = synth.base("c2", n)
        truth = exact10(X, Q)
        recs, searches = [], []
        for b in range(BUILDS):
            p = oracle_py.params(**{**FLAGS, "nthreads": threads})
            rows, ep, width, csv = ref.build(oracle_py.KCNA_NSG, X, p, nthreads=threads)
            r = oracle_py.parse_run_csv(csv)
            rec = np.full(32, np.nan, np.float64)
            rec[: len(r["recall"])] = r["recall"]
            recs.append(rec)
            W = max(len(x) for x in rows)
            g = np.full((n, W), 0xFFFFFFFF, np.uint32)
            deg = np.zeros(n, np.uint32)
            for i, x in enumerate(rows):
                g[i, : len(x)] = x
                deg[i] = len(x)
            sr = []
            for L in BEAMS:
                init = np.broadcast_to(start_nodes(n, ep, L), (NQ, L)).copy()
                found, _ = ref.beam_search(X, g, deg, Q, init, L, 10)
                hit = sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth))
                sr.append(hit / (10.0 * NQ))
            searches.append(sr)
            print(f"n={n} build {b}: recall {np.round(rec[~np.isnan(rec)], 5).tolist()} "
                  f"search@10 {dict(zip(BEAMS, np.round(sr, 4).tolist()))}", flush=True)
        out[f"recall_{n}"] = np.asarray(recs)
        out[f"search10_{n}"] = np.asarray(searches)
    np.savez_compressed(os.path.join(HERE, "ref_quality_c2.npz"), **out)


if __name__ == "__main__":
    main()
