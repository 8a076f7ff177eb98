"""Generates tests/golden/ref_cli_c1.npz from the reference itself.

The reference's own builds (oracle/_ref/libkcna_ref.so, compiled from its
sources by oracle/build_ref.sh) of C1 data (20,000 x 32, seeded generator),
with the flags the command-line tests use, scored by the tests' host searcher
(tests/graph_search.py) on 1,000 seeded queries:
  * recall@10 of two builds each of the NSG, tau-MNG and alpha-PG indexes (buildFast*, beam 60
    from the entry point plus 59 seeded random nodes);
  * recall@10 of the layered HNSW (ef 60 after the greedy descent) and of the
    one-level NSW (ef 60 from the entry point plus 59 seeded random nodes),
    built the way the fasthnsw / fastnsw tools do;
  * the HNSW level assignment (Matrix::getlevel): storage order -> file row
    and the node count per level.

Usage: python tests/golden/make_golden_cli.py   (needs oracle/_ref built here)
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)):
    sys.path.insert(0, p)

import oracle_py  # noqa: E402
from fastkcna_gb300 import index_io, synth  # noqa: E402
from graph_search import beam_search, hnsw_search, seeded_entries  # noqa: E402

N, NQ = 20000, 1000
BUILDS = 2  # the reference's builds differ with OpenMP timing: the tests allow the range they span
PARAMS = dict(K=100, L=100, S=10, R=100, iterations=6, search_L=40, nsg_R=32, search_K=100, massq_S=10,
              angle=60.0, tau=0.1)


def truth(X, Q, k=10):
    d = ((Q[:, None, :].astype(np.float64) - X[None, :, :]) ** 2).sum(-1)
    return np.argsort(d, axis=1, kind="stable")[:, :k]


def recall(found, t):
    return float(np.mean([len(set(f[:10].tolist()) & set(g[:10].tolist())) / 10 for f, g in zip(found, t)]))


def main():
    ref = oracle_py.Reference()
    X = synth.base("c1", N)
    Q = synth.queries("c1", NQ)
    T = truth(X, Q)
    p = oracle_py.params(**PARAMS)
    out = {}
    out["nq"] = np.int32(NQ)
    for kind, tag in ((1, "nsg"), (3, "taumng"), (4, "alphapg")):
        recs = []
        for _ in range(BUILDS):
            rows, ep, width, _ = ref.build(kind, X, p, nthreads=8)
            rows = [np.asarray(r, np.int64) for r in rows]
            start = seeded_entries(N, ep, 60)
            recs.append(recall([beam_search(X, rows, start, q, 60, 10) for q in Q], T))
        out[f"recall_{tag}"] = np.asarray(recs)
        print(tag, recs)
    with tempfile.TemporaryDirectory() as td:
        for single, tag in ((False, "hnsw"), (True, "nsw")):
            recs = []
            for _ in range(BUILDS):
                path = os.path.join(td, tag + ".bin")
                ref.build_hnsw(X, p, path, single_level=single, nthreads=8)
                idx = index_io.read_hnswlib(path)
                recs.append(recall(hnsw_search(idx, Q, 60, 10, extra_entries=59 if single else 0), T))
            out[f"recall_{tag}"] = np.asarray(recs)
            out[f"maxlevel_{tag}"] = idx["maxlevel"]
            print(tag, recs, idx["maxlevel"])
    d2f, pn = ref.getlevel(N, PARAMS["nsg_R"], p.seed)
    out["levels_data2file"], out["levels_points_num"] = d2f, pn
    np.savez_compressed(os.path.join(HERE, "ref_cli_c1.npz"), **out)


if __name__ == "__main__":
    main()
