"""TEST INFRASTRUCTURE: ctypes bindings of the oracle restatement
(oracle/libkcna_oracle.so) and of the reference harness
(oracle/_ref/libkcna_ref.so, present only where the reference sources were
available at build time).  Only tests, the smoke check and the bench's CPU
baseline import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libkcna_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libkcna_ref.so")

KCNA_NSG, KCNA_HNSW_LAYER, KCNA_TAUMNG, KCNA_ALPHAPG, KCNA_CAGRA = 1, 2, 3, 4, 5
MAX_ITERS, MAX_LOOPS = 64, 16


class Params(C.Structure):
    _fields_ = [
        (n, C.c_uint32)
        for n in ("K", "L", "S", "R", "iterations", "controls", "seed", "nthreads")
    ] + [("delta", C.c_float), ("recall", C.c_float)] + [
        (n, C.c_uint32) for n in ("nsg_R", "search_L", "search_K", "step", "massq_S", "loop_i")
    ] + [("tau", C.c_float), ("angle", C.c_float)] + [
        ("screen", C.c_uint32), ("learned_seed", C.c_uint32), ("verbosity", C.c_uint32),
        ("refine", C.c_uint32), ("reserved", C.c_uint32 * 4),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint32), ("stop_condition", C.c_uint32), ("maxl", C.c_uint32), ("loops", C.c_uint32),
        ("iter_recall", C.c_float * MAX_ITERS), ("iter_delta", C.c_float * MAX_ITERS),
        ("iter_time", C.c_double * MAX_ITERS), ("iter_cand_overflow", C.c_uint64 * MAX_ITERS),
        ("loop_recall", C.c_float * (MAX_LOOPS + 1)),
        ("prune_time", C.c_double * MAX_LOOPS), ("inter_time", C.c_double * MAX_LOOPS),
        ("tree_grow_time", C.c_double * MAX_LOOPS), ("buildnsg_time", C.c_double * MAX_LOOPS),
        ("search_time", C.c_double * MAX_LOOPS), ("con_time", C.c_double * MAX_LOOPS),
        ("nndescent_time", C.c_double), ("total_time", C.c_double),
        ("n_comps", C.c_uint64), ("prune_comps", C.c_uint64), ("bridge_comps", C.c_uint64),
        ("screened_pairs", C.c_uint64), ("rescored_pairs", C.c_uint64),
        ("ep", C.c_uint32), ("width", C.c_uint32), ("aod", C.c_uint32),
        ("min_degree", C.c_uint32), ("max_degree", C.c_uint32), ("rev_overflow", C.c_uint32), ("reserved", C.c_uint32 * 2),
        ("phase_ms", C.c_double * 12), ("phase_launches", C.c_uint64 * 12),
        ("join_rows", C.c_uint64), ("cand_emitted", C.c_uint64), ("cand_merged", C.c_uint64),
        ("pool_entries_merged", C.c_uint64), ("tree_attached", C.c_uint64),
        ("iter_join_ms", C.c_double * MAX_ITERS), ("iter_merge_ms", C.c_double * MAX_ITERS),
        ("iter_cand", C.c_uint64 * MAX_ITERS), ("iter_inserted", C.c_uint64 * MAX_ITERS),
        ("seed_train_ms", C.c_double), ("seed_total_ms", C.c_double), ("seed_loss_first", C.c_float),
        ("seed_loss_last", C.c_float), ("seed_input_scale", C.c_float), ("seed_recall", C.c_float),
        ("seed_comps", C.c_uint64), ("bf16_rows", C.c_uint32), ("gram_tc", C.c_uint32),
        ("prune_tc", C.c_uint32), ("prune_exact", C.c_uint64), ("prune_skipped", C.c_uint64),
    ]


def params(**kw) -> Params:
    """Reference defaults (src/kgraph.h:12-40) overridden by keywords."""
    p = Params()
    d = dict(K=25, L=100, S=10, R=100, iterations=30, controls=100, seed=2024, nthreads=40, delta=0.002,
             recall=0.95, nsg_R=50, search_L=40, search_K=500, step=10, massq_S=10, loop_i=2, tau=0.0,
             angle=60.0, screen=0, learned_seed=0, verbosity=0, refine=0)
    d.update(kw)
    for k, v in d.items():
        setattr(p, k, v)
    return p


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def build_ref() -> bool:
    """Builds oracle/_ref when the reference sources are present."""
    r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True)
    return r.returncode == 0


_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def _u32(x):
    return np.ascontiguousarray(x, dtype=np.uint32)


class _Lib:
    def __init__(self, path, prefix):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.prefix = prefix

    def fn(self, name):
        f = getattr(self.lib, self.prefix + name)
        f.restype = C.c_int
        return f


class Oracle(_Lib):
    """The CPU restatement.  Arrays are numpy; X is (n, d) float32 C-contiguous."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        super().__init__(path, "kcnao_")
        self.lib.kcnao_l2.restype = C.c_float

    def l2(self, a, b):
        a, b = _f32(a), _f32(b)
        return float(self.lib.kcnao_l2(_ptr(a), _ptr(b), C.c_uint32(a.size)))

    def knn(self, X, ids, k, nthreads=0):
        X, ids = _f32(X), _u32(ids)
        n, d = X.shape
        oi = np.empty((ids.size, k), np.uint32)
        od = np.empty((ids.size, k), np.float32)
        rc = self.fn("knn")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), _ptr(ids), C.c_uint32(ids.size),
                            C.c_uint32(k), _ptr(oi), _ptr(od), C.c_int(nthreads))
        assert rc == 0, rc
        return oi, od

    def knn_queries(self, X, Q, k, nthreads=0):
        X, Q = _f32(X), _f32(Q)
        n, d = X.shape
        oi = np.empty((Q.shape[0], k), np.uint32)
        od = np.empty((Q.shape[0], k), np.float32)
        rc = self.fn("knn_queries")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), _ptr(Q), C.c_uint64(d),
                                    C.c_uint32(Q.shape[0]), C.c_uint32(k), _ptr(oi), _ptr(od), C.c_int(nthreads))
        assert rc == 0, rc
        return oi, od

    def pool_insert_seq(self, ids, dists, flags, L, cap, radius, cid, cd):
        ids = _u32(np.resize(ids, cap + 1)).copy()
        dists = _f32(np.resize(dists, cap + 1)).copy()
        flags = np.ascontiguousarray(np.resize(flags, cap + 1), dtype=np.uint8).copy()
        Lc = C.c_uint32(L)
        rad = C.c_float(radius)
        cid, cd = _u32(cid), _f32(cd)
        ret = np.empty(cid.size, np.uint32)
        self.fn("pool_insert_seq")(_ptr(ids), _ptr(dists), _ptr(flags), C.byref(Lc), C.c_uint32(cap), C.byref(rad),
                                   _ptr(cid), _ptr(cd), C.c_uint32(cid.size), _ptr(ret))
        L = Lc.value
        return ids[:L], dists[:L], flags[:L], L, rad.value, ret

    def _graph_call(self, name, kind, X, p, pid, pd, pcnt, width, nthreads):
        X, pid, pd, pcnt = _f32(X), _u32(pid), _f32(pd), _u32(pcnt)
        n, d = X.shape
        cap = pid.shape[1]
        gi = np.empty((n, width), np.uint32)
        gd = np.empty((n, width), np.float32)
        deg = np.empty(n, np.uint32)
        rc = self.fn(name)(C.c_int(kind), _ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p),
                           _ptr(pid), _ptr(pd), _ptr(pcnt), C.c_uint32(cap), _ptr(gi), _ptr(gd), _ptr(deg),
                           C.c_uint32(width), C.c_int(nthreads))
        assert rc == 0, rc
        return gi, gd, deg

    def prune(self, kind, X, p, pid, pd, pcnt, width, nthreads=0):
        return self._graph_call("prune", kind, X, p, pid, pd, pcnt, width, nthreads)

    def link(self, kind, X, p, pid, pd, pcnt, width, nthreads=0):
        return self._graph_call("link", kind, X, p, pid, pd, pcnt, width, nthreads)

    def pool_search(self, X, p, pid, pd, pcnt, g_ids, g_deg, loopcount, nthreads=0):
        """inSearch of loop `loopcount` on the given pools over the given graph:
        (pool ids, dists, counts, distance evaluations)."""
        X, pid, pd, pcnt, g_ids, g_deg = _f32(X), _u32(pid), _f32(pd), _u32(pcnt), _u32(g_ids), _u32(g_deg)
        n, d = X.shape
        cap = pid.shape[1]
        oi = np.empty((n, cap), np.uint32)
        od = np.empty((n, cap), np.float32)
        oc = np.empty(n, np.uint32)
        cc = C.c_uint64(0)
        rc = self.fn("pool_search")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), _ptr(pid),
                                    _ptr(pd), _ptr(pcnt), C.c_uint32(cap), _ptr(g_ids), _ptr(g_deg),
                                    C.c_uint32(g_ids.shape[1]), C.c_uint32(loopcount), _ptr(oi), _ptr(od), _ptr(oc),
                                    C.byref(cc), C.c_int(nthreads))
        assert rc == 0, rc
        return oi, od, oc, cc.value

    def beam_search(self, X, g_ids, g_deg, Q, init_ids, L, k, nthreads=0):
        X, g_ids, g_deg, Q, init_ids = _f32(X), _u32(g_ids), _u32(g_deg), _f32(Q), _u32(init_ids)
        n, d = X.shape
        m = Q.shape[0]
        oi = np.empty((m, k), np.uint32)
        od = np.empty((m, k), np.float32)
        rc = self.fn("beam_search")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), _ptr(g_ids), _ptr(g_deg),
                                    C.c_uint32(g_ids.shape[1]), _ptr(Q), C.c_uint64(d), C.c_uint32(m),
                                    _ptr(init_ids), C.c_uint32(L), C.c_uint32(k), _ptr(oi), _ptr(od),
                                    C.c_int(nthreads))
        assert rc == 0, rc
        return oi, od

    def nndescent(self, X, p, cap=None, nthreads=0):
        X = _f32(X)
        n, d = X.shape
        st = Stats()
        cap = cap or max(p.L, p.K, p.search_L, p.search_K)
        pid = np.empty((n, cap), np.uint32)
        pd = np.empty((n, cap), np.float32)
        pc = np.empty(n, np.uint32)
        rc = self.fn("nndescent")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), C.byref(st),
                                  _ptr(pid), _ptr(pd), _ptr(pc), C.c_uint32(cap), C.c_int(nthreads))
        assert rc == 0, rc
        return pid, pd, pc, st

    def build(self, kind, X, p, width=None, use_prune2=True, nthreads=0):
        X = _f32(X)
        n, d = X.shape
        st = Stats()
        width = width or 2 * p.nsg_R + 64
        gi = np.empty((n, width), np.uint32)
        deg = np.empty(n, np.uint32)
        rc = self.fn("build")(C.c_int(kind), _ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p),
                              C.byref(st), _ptr(gi), _ptr(deg), C.c_uint32(width), C.c_int(int(use_prune2)),
                              C.c_int(nthreads))
        assert rc == 0, rc
        return gi, deg, st


class Reference(_Lib):
    """The reference's own code (compiled by oracle/build_ref.sh)."""

    def __init__(self, path=REF_SO, trap_faults=True):
        super().__init__(path, "kref_")
        self.lib.kref_l2.restype = C.c_float
        if trap_faults:  # a crash in the reference's code exits 70 with a stack trace
            self.lib.kref_trap_faults()

    @staticmethod
    def available(path=REF_SO) -> bool:
        return os.path.exists(path)

    def l2(self, a, b):
        a = np.zeros(((a.size + 7) // 8) * 8, np.float32) + np.pad(_f32(a), (0, (-a.size) % 8))
        b = np.zeros(((b.size + 7) // 8) * 8, np.float32) + np.pad(_f32(b), (0, (-b.size) % 8))
        return float(self.lib.kref_l2(_ptr(a), _ptr(b), C.c_uint32(a.size)))

    def linear_search(self, X, ids, k):
        X, ids = _f32(X), _u32(ids)
        n, d = X.shape
        oi = np.empty((ids.size, k), np.uint32)
        od = np.empty((ids.size, k), np.float32)
        self.fn("linear_search")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), _ptr(ids),
                                 C.c_uint32(ids.size), C.c_uint32(k), _ptr(oi), _ptr(od))
        return oi, od

    def nndescent(self, X, p, cap=None, nthreads=8):
        X = _f32(X)
        n, d = X.shape
        cap = cap or max(p.L, p.K, p.search_L, p.search_K)
        pid = np.empty((n, cap), np.uint32)
        pd = np.empty((n, cap), np.float32)
        pc = np.empty(n, np.uint32)
        rec = np.zeros(MAX_ITERS, np.float32)
        iters = C.c_uint32(0)
        fin = C.c_float(0)
        self.fn("nndescent")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), C.c_int(nthreads),
                             _ptr(pid), _ptr(pd), _ptr(pc), C.c_uint32(cap), _ptr(rec), C.byref(iters),
                             C.byref(fin))
        return pid, pd, pc, rec[: iters.value].copy(), fin.value

    def _graph_call(self, name, kind, X, p, pid, pd, pcnt, width):
        X, pid, pd, pcnt = _f32(X), _u32(pid), _f32(pd), _u32(pcnt)
        n, d = X.shape
        cap = pid.shape[1]
        gi = np.empty((n, width), np.uint32)
        gd = np.empty((n, width), np.float32)
        deg = np.empty(n, np.uint32)
        self.fn(name)(C.c_int(kind), _ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), _ptr(pid),
                      _ptr(pd), _ptr(pcnt), C.c_uint32(cap), _ptr(gi), _ptr(gd), _ptr(deg), C.c_uint32(width))
        return gi, gd, deg

    def prune(self, kind, X, p, pid, pd, pcnt, width):
        return self._graph_call("prune", kind, X, p, pid, pd, pcnt, width)

    def link(self, kind, X, p, pid, pd, pcnt, width):
        return self._graph_call("link", kind, X, p, pid, pd, pcnt, width)

    def pool_search(self, X, p, pid, pd, pcnt, g_ids, g_deg, loopcount, nthreads=8):
        X, pid, pd, pcnt, g_ids, g_deg = _f32(X), _u32(pid), _f32(pd), _u32(pcnt), _u32(g_ids), _u32(g_deg)
        n, d = X.shape
        cap = pid.shape[1]
        oi = np.empty((n, cap), np.uint32)
        od = np.empty((n, cap), np.float32)
        oc = np.empty(n, np.uint32)
        scan = C.c_float(0)
        self.fn("pool_search")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), _ptr(pid), _ptr(pd),
                               _ptr(pcnt), C.c_uint32(cap), _ptr(g_ids), _ptr(g_deg), C.c_uint32(g_ids.shape[1]),
                               C.c_uint32(loopcount), C.c_int(nthreads), _ptr(oi), _ptr(od), _ptr(oc), C.byref(scan))
        return oi, od, oc, scan.value

    def refine(self, X, p, pid, pd, pcnt, g_ids, g_deg, loop, pflags=None, g_old=None, g_old_deg=None, nthreads=1):
        """UpdateNhoods + BridgeView of P2K loop `loop` (harness kref_refine):
        returns (pool ids, dists, counts, flags, isnew flags of g, comps)."""
        X, pid, pd, pcnt, g_ids, g_deg = _f32(X), _u32(pid), _f32(pd), _u32(pcnt), _u32(g_ids), _u32(g_deg)
        n, d = X.shape
        cap, W = pid.shape[1], g_ids.shape[1]
        pf = None if pflags is None else np.ascontiguousarray(pflags, dtype=np.uint8)
        go = None if g_old is None else _u32(g_old)
        god = None if g_old_deg is None else _u32(g_old_deg)
        oi = np.empty((n, cap), np.uint32)
        od = np.empty((n, cap), np.float32)
        oc = np.empty(n, np.uint32)
        of = np.empty((n, cap), np.uint8)
        isnew = np.empty((n, W), np.uint8)
        comps = C.c_uint64(0)
        self.fn("refine")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p), _ptr(pid), _ptr(pd),
                          _ptr(pcnt), _ptr(pf), C.c_uint32(cap), _ptr(g_ids), _ptr(g_deg), _ptr(go), _ptr(god),
                          C.c_uint32(W), C.c_uint32(loop), C.c_int(nthreads), _ptr(oi), _ptr(od), _ptr(oc), _ptr(of),
                          _ptr(isnew), C.byref(comps))
        return oi, od, oc, of, isnew, comps.value

    def beam_search(self, X, g_ids, g_deg, Q, init_ids, L, k):
        X, g_ids, g_deg, Q, init_ids = _f32(X), _u32(g_ids), _u32(g_deg), _f32(Q), _u32(init_ids)
        n, d = X.shape
        m = Q.shape[0]
        oi = np.empty((m, k), np.uint32)
        od = np.empty((m, k), np.float32)
        self.fn("beam_search")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), _ptr(g_ids), _ptr(g_deg),
                               C.c_uint32(g_ids.shape[1]), _ptr(Q), C.c_uint64(d), C.c_uint32(m), _ptr(init_ids),
                               C.c_uint32(L), C.c_uint32(k), _ptr(oi), _ptr(od))
        return oi, od

    def getlevel(self, n, M, seed, max_levels=64):
        """hnsw_dataload's level assignment: (data2file, points_num)."""
        d2f = np.empty(n, np.int32)
        pn = np.empty(max_levels, np.int32)
        nl = C.c_uint32(0)
        rc = self.fn("getlevel")(C.c_uint32(n), C.c_uint32(M), C.c_uint32(seed), _ptr(d2f), _ptr(pn),
                                 C.c_uint32(max_levels), C.byref(nl))
        assert rc == 0, rc
        return d2f, pn[: nl.value].copy()

    def build_hnsw(self, X, p, path, single_level=False, nthreads=8, quiet=True):
        """Layered HNSW build (fasthnsw / fastnsw orchestration) into an hnswlib file."""
        X = _f32(X)
        n, d = X.shape
        rc = self.fn("build_hnsw")(_ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p),
                                   C.c_int(nthreads), C.c_int(int(single_level)), path.encode(), C.c_int(int(quiet)))
        assert rc == 0, rc

    def build(self, kind, X, p, nthreads=8, quiet=True):
        """Runs buildFast* and returns (graph rows as lists, ep, width, csv text)."""
        X = _f32(X)
        n, d = X.shape
        with tempfile.TemporaryDirectory() as td:
            ip, cp = os.path.join(td, "g.nsg"), os.path.join(td, "r.csv")
            self.fn("build")(C.c_int(kind), _ptr(X), C.c_uint64(d), C.c_uint32(n), C.c_uint32(d), C.byref(p),
                             C.c_int(nthreads), ip.encode(), cp.encode(), C.c_int(int(quiet)))
            g = read_nsg(ip)
            csv = open(cp).read() if os.path.exists(cp) else ""
        return g + (csv,)


def parse_run_csv(text):
    """Rows of the reference's run CSV (SaveResult, src/kgraph.cpp:1725-1807):
    {"kgraph time": [...], "recall": [...], "con time": [...], ...} as floats,
    plus "params" (the PG_type,K,L,... row as a dict)."""
    out = {}
    lines = [ln for ln in text.splitlines() if ln.strip()]
    for i, ln in enumerate(lines):
        f = ln.split(",")
        if f[0] == "PG_type" and i + 1 < len(lines):
            out["params"] = dict(zip(f, lines[i + 1].split(",")))
            continue
        vals = []
        for x in f[1:]:
            try:
                vals.append(float(x))
            except ValueError:
                pass
        if f[0] and not f[0][0].isdigit():
            out[f[0]] = vals
    return out


def read_nsg(path):
    """NSG/efanna file (SaveNsg, src/kgraph.cpp:1704-1724): u32 width, u32 ep,
    then per node u32 GK + GK ids.  Returns (list of id arrays, ep, width)."""
    raw = np.fromfile(path, dtype=np.uint32)
    width, ep = int(raw[0]), int(raw[1])
    rows, i = [], 2
    while i < raw.size:
        k = int(raw[i])
        rows.append(raw[i + 1: i + 1 + k].copy())
        i += 1 + k
    return rows, ep, width
