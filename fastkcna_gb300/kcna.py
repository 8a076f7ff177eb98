"""ctypes binding of the C ABI in include/kcna.h (libkcna.so, built in-tree).

This is the Python face of the drop-in boundary: numpy arrays in, numpy arrays
out, status codes turned into the exception types of the reference
(kgraph::invalid_argument -> ValueError, kgraph::io_error -> IOError,
kgraph::runtime_error -> RuntimeError; src/kgraph.h:363-376).  There is no
fallback: when the CUDA library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkcna.so")

NSG, HNSW_LAYER, TAUMNG, ALPHAPG, CAGRA = 1, 2, 3, 4, 5
KINDS = {"nsg": NSG, "hnsw": HNSW_LAYER, "taumng": TAUMNG, "alphapg": ALPHAPG, "cagra": CAGRA}
SCREEN_FP32, SCREEN_BF16 = 0, 1
MAX_ITERS, MAX_LOOPS, NUM_PHASES = 64, 16, 12
PHASES = ["join", "merge", "sample", "prune", "link", "p2k", "ep", "tree", "controls", "init", "other", "spare"]
STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "cuda error", 4: "timeout", 5: "io error",
          6: "bad call order", 7: "limit exceeded"}


class KcnaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"kcna {STATUS.get(status, status)}: {msg}")
        self.status = status


class KcnaArgError(KcnaError, ValueError):
    pass


class KcnaIOError(KcnaError, IOError):
    pass


class Params(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("K", "L", "S", "R", "iterations", "controls", "seed", "nthreads")] + [
        ("delta", C.c_float), ("recall", C.c_float)] + [
        (n, C.c_uint32) for n in ("nsg_R", "search_L", "search_K", "step", "massq_S", "loop_i")] + [
        ("tau", C.c_float), ("angle", C.c_float), ("screen", C.c_uint32), ("learned_seed", C.c_uint32),
        ("verbosity", C.c_uint32), ("refine", C.c_uint32), ("reserved", C.c_uint32 * 4)]


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
        ("phase_ms", C.c_double * NUM_PHASES), ("phase_launches", C.c_uint64 * NUM_PHASES),
        ("join_rows", C.c_uint64), ("cand_emitted", C.c_uint64), ("cand_merged", C.c_uint64),
        ("pool_entries_merged", C.c_uint64), ("tree_attached", C.c_uint64),
        ("iter_join_ms", C.c_double * MAX_ITERS), ("iter_merge_ms", C.c_double * MAX_ITERS),
        ("iter_cand", C.c_uint64 * MAX_ITERS), ("iter_inserted", C.c_uint64 * MAX_ITERS),
        ("seed_train_ms", C.c_double), ("seed_total_ms", C.c_double), ("seed_loss_first", C.c_float),
        ("seed_loss_last", C.c_float), ("seed_input_scale", C.c_float), ("seed_recall", C.c_float),
        ("seed_comps", C.c_uint64), ("bf16_rows", C.c_uint32), ("gram_tc", C.c_uint32), ("prune_tc", C.c_uint32),
        ("prune_exact", C.c_uint64), ("prune_skipped", C.c_uint64)]

    def as_dict(self):
        it = self.iterations
        lp = self.loops
        return dict(iterations=it, stop_condition=self.stop_condition, maxl=self.maxl, loops=lp,
                    iter_recall=list(self.iter_recall[:it]), iter_delta=list(self.iter_delta[:it]),
                    iter_time=list(self.iter_time[:it]), iter_cand_overflow=list(self.iter_cand_overflow[:it]),
                    loop_recall=list(self.loop_recall[:max(lp, 1)]), prune_time=list(self.prune_time[:lp]),
                    tree_grow_time=list(self.tree_grow_time[:lp]), search_time=list(self.search_time[:max(lp - 1, 0)]),
                    con_time=list(self.con_time[:lp]), nndescent_time=self.nndescent_time,
                    total_time=self.total_time, n_comps=self.n_comps, prune_comps=self.prune_comps,
                    bridge_comps=self.bridge_comps, screened_pairs=self.screened_pairs,
                    rescored_pairs=self.rescored_pairs, ep=self.ep, width=self.width, aod=self.aod,
                    min_degree=self.min_degree, max_degree=self.max_degree, rev_overflow=self.rev_overflow,
                    phase_ms={PHASES[i]: self.phase_ms[i] for i in range(NUM_PHASES)},
                    phase_launches={PHASES[i]: int(self.phase_launches[i]) for i in range(NUM_PHASES)},
                    join_rows=self.join_rows, cand_emitted=self.cand_emitted, cand_merged=self.cand_merged,
                    pool_entries_merged=self.pool_entries_merged, tree_attached=self.tree_attached,
                    iter_join_ms=list(self.iter_join_ms[:it]), iter_merge_ms=list(self.iter_merge_ms[:it]),
                    iter_cand=list(self.iter_cand[:it]), iter_inserted=list(self.iter_inserted[:it]),
                    seed_train_ms=self.seed_train_ms, seed_total_ms=self.seed_total_ms,
                    seed_loss_first=self.seed_loss_first, seed_loss_last=self.seed_loss_last,
                    seed_input_scale=self.seed_input_scale, seed_recall=self.seed_recall,
                    seed_comps=self.seed_comps, bf16_rows=self.bf16_rows, gram_tc=self.gram_tc, prune_tc=self.prune_tc,
                    prune_exact=self.prune_exact, prune_skipped=self.prune_skipped)


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(path)
    P, U32, U64, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "kcna_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
        "kcna_destroy": ([P], None),
        "kcna_last_error": ([P], C.c_char_p),
        "kcna_version": ([], C.c_char_p),
        "kcna_params_default": ([C.POINTER(Params)], None),
        "kcna_upload": ([P, P, U32, U32, U64], C.c_int),
        "kcna_upload_device": ([P, P, U32, U32, U64], C.c_int),
        "kcna_set_size": ([P, U32], C.c_int),
        "kcna_knn_exact": ([P, P, U32, U32, P, P], C.c_int),
        "kcna_knn_queries": ([P, P, U32, U64, U32, P, P], C.c_int),
        "kcna_build": ([P, C.POINTER(Params), C.c_int, C.POINTER(Stats)], C.c_int),
        "kcna_nndescent": ([P, C.POINTER(Params), C.POINTER(Stats)], C.c_int),
        "kcna_get_graph": ([P, P, P, P, P], C.c_int),
        "kcna_pool_capacity": ([P, C.POINTER(U32)], C.c_int),
        "kcna_get_pools": ([P, P, P, P, U32], C.c_int),
        "kcna_set_pools": ([P, C.POINTER(Params), P, P, P, U32], C.c_int),
        "kcna_prune": ([P, C.POINTER(Params), C.c_int], C.c_int),
        "kcna_link": ([P, C.POINTER(Params), C.c_int], C.c_int),
        "kcna_set_graph": ([P, P, P, U32, U32], C.c_int),
        "kcna_search": ([P, P, U32, U64, P, U32, U32, P, P], C.c_int),
        "kcna_kernel_launches": ([P], U64),
        "kcna_stream": ([P], C.c_void_p),
        "kcna_write_nsg": ([P, C.c_char_p], C.c_int),
        "kcna_write_nsg_async": ([P, C.c_char_p], C.c_int),
        "kcna_wait_writes": ([P], C.c_int),
        "kcna_upload_lshkit": ([P, C.c_char_p], C.c_int),
        "kcna_pool_search": ([P, C.POINTER(Params), U32, C.POINTER(U64)], C.c_int),
        "kcna_refine_pools": ([P, C.POINTER(Params), U32, C.POINTER(U64)], C.c_int),
        "kcna_get_edge_isnew": ([P, P], C.c_int),
    }
    for name, (argt, rest) in sig.items():
        f = getattr(lib, name)
        f.argtypes = argt
        f.restype = rest
    _lib = lib
    return lib


def params(**kw) -> Params:
    """IndexParams defaults (src/kgraph.h:12-40) overridden by keywords."""
    lib = load_library()
    p = Params()
    lib.kcna_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KcnaArgError(1, f"unknown parameter {k}")
        setattr(p, k, v)
    return p


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def _u32(x):
    return np.ascontiguousarray(x, dtype=np.uint32)


class Index:
    """One build context on one CUDA device (the KGraph object of the reference)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.kcna_create(C.byref(h), device)
        if rc != 0:
            raise KcnaError(rc, f"kcna_create(device={device}) failed")
        self.h = h
        self.n = 0
        self.d = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.kcna_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc == 0:
            return
        msg = (self.lib.kcna_last_error(self.h) or b"").decode()
        if rc == 1:
            raise KcnaArgError(rc, msg)
        if rc == 5:
            raise KcnaIOError(rc, msg)
        raise KcnaError(rc, msg)

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.lib.kcna_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.kcna_kernel_launches(self.h))

    def upload(self, X) -> None:
        """Host rows (n, d) float32 -> device."""
        X = _f32(X)
        self._check(self.lib.kcna_upload(self.h, _ptr(X), X.shape[0], X.shape[1], X.strides[0]))
        self.n, self.d = X.shape

    def upload_device(self, ptr: int, n: int, d: int, stride_bytes: int) -> None:
        """Rows already in device memory of this context's device."""
        self._check(self.lib.kcna_upload_device(self.h, C.c_void_p(ptr), n, d, stride_bytes))
        self.n, self.d = n, d

    def set_size(self, n_prefix: int) -> None:
        self._check(self.lib.kcna_set_size(self.h, n_prefix))
        self.n = min(n_prefix, self.n)

    def knn_exact(self, ids, k: int):
        ids = _u32(ids)
        oi = np.empty((ids.size, k), np.uint32)
        od = np.empty((ids.size, k), np.float32)
        self._check(self.lib.kcna_knn_exact(self.h, _ptr(ids), ids.size, k, _ptr(oi), _ptr(od)))
        return oi, od

    def knn_queries(self, Q, k: int):
        Q = _f32(Q)
        oi = np.empty((Q.shape[0], k), np.uint32)
        od = np.empty((Q.shape[0], k), np.float32)
        self._check(self.lib.kcna_knn_queries(self.h, _ptr(Q), Q.shape[0], Q.strides[0], k, _ptr(oi), _ptr(od)))
        return oi, od

    def build(self, kind="nsg", p: Params | None = None, **kw) -> dict:
        p = p or params(**kw)
        st = Stats()
        self._check(self.lib.kcna_build(self.h, C.byref(p), KINDS.get(kind, kind), C.byref(st)))
        return st.as_dict()

    def nndescent(self, p: Params | None = None, **kw) -> dict:
        p = p or params(**kw)
        st = Stats()
        self._check(self.lib.kcna_nndescent(self.h, C.byref(p), C.byref(st)))
        return st.as_dict()

    def graph(self):
        """(ids (n, width) padded with 0xFFFFFFFF, degrees (n,), ep)."""
        w = C.c_uint32()
        ep = C.c_uint32()
        self._check(self.lib.kcna_get_graph(self.h, None, None, C.byref(ep), C.byref(w)))
        ids = np.empty((self.n, w.value), np.uint32)
        deg = np.empty(self.n, np.uint32)
        self._check(self.lib.kcna_get_graph(self.h, _ptr(ids), _ptr(deg), C.byref(ep), C.byref(w)))
        return ids, deg, int(ep.value)

    def pools(self):
        cap = C.c_uint32()
        self._check(self.lib.kcna_pool_capacity(self.h, C.byref(cap)))
        c = cap.value
        ids = np.empty((self.n, c), np.uint32)
        d = np.empty((self.n, c), np.float32)
        cnt = np.empty(self.n, np.uint32)
        self._check(self.lib.kcna_get_pools(self.h, _ptr(ids), _ptr(d), _ptr(cnt), c))
        return ids, d, cnt

    def pool_search(self, loopcount: int, p: Params | None = None, **kw) -> int:
        """Per-node pool search of loop `loopcount` (inSearch) over the current
        graph; returns the distance evaluations."""
        p = p or params(**kw)
        cc = C.c_uint64(0)
        self._check(self.lib.kcna_pool_search(self.h, C.byref(p), C.c_uint32(loopcount), C.byref(cc)))
        return int(cc.value)

    def refine(self, loopcount: int, p: Params | None = None, **kw) -> int:
        """UpdateNhoods + the pool refinement of loop `loopcount` (BridgeView,
        or the pool search when p.refine says so) over the current graph, as a
        build runs it between prune loops; returns the distance evaluations."""
        p = p or params(**kw)
        cc = C.c_uint64(0)
        self._check(self.lib.kcna_refine_pools(self.h, C.byref(p), C.c_uint32(loopcount), C.byref(cc)))
        return int(cc.value)

    def edge_isnew(self):
        """isnew flag of every graph edge (n, width) uint8, as UpdateNhoods set it."""
        w = C.c_uint32()
        ep = C.c_uint32()
        self._check(self.lib.kcna_get_graph(self.h, None, None, C.byref(ep), C.byref(w)))
        out = np.empty((self.n, w.value), np.uint8)
        self._check(self.lib.kcna_get_edge_isnew(self.h, _ptr(out)))
        return out

    def set_pools(self, ids, dists, counts, p: Params | None = None, **kw):
        p = p or params(**kw)
        ids, dists, counts = _u32(ids), _f32(dists), _u32(counts)
        self._check(self.lib.kcna_set_pools(self.h, C.byref(p), _ptr(ids), _ptr(dists), _ptr(counts),
                                            ids.shape[1]))

    def prune(self, kind="nsg", p: Params | None = None, **kw):
        p = p or params(**kw)
        self._check(self.lib.kcna_prune(self.h, C.byref(p), KINDS.get(kind, kind)))

    def link(self, kind="nsg", p: Params | None = None, **kw):
        p = p or params(**kw)
        self._check(self.lib.kcna_link(self.h, C.byref(p), KINDS.get(kind, kind)))

    def set_graph(self, ids, degrees, ep: int):
        ids, degrees = _u32(ids), _u32(degrees)
        self._check(self.lib.kcna_set_graph(self.h, _ptr(ids), _ptr(degrees), ids.shape[1], ep))

    def search(self, Q, L: int, k: int, init_ids=None):
        Q = _f32(Q)
        m = Q.shape[0]
        init = None if init_ids is None else _u32(init_ids)
        oi = np.empty((m, k), np.uint32)
        od = np.empty((m, k), np.float32)
        self._check(self.lib.kcna_search(self.h, _ptr(Q), m, Q.strides[0], _ptr(init), L, k, _ptr(oi), _ptr(od)))
        return oi, od

    def write_nsg(self, path: str):
        self._check(self.lib.kcna_write_nsg(self.h, path.encode()))

    def write_nsg_async(self, path: str):
        """Snapshot the graph and write the NSG file on a host thread."""
        self._check(self.lib.kcna_write_nsg_async(self.h, path.encode()))

    def wait_writes(self):
        self._check(self.lib.kcna_wait_writes(self.h))

    def upload_lshkit(self, path: str):
        """Rows straight from an lshkit file (mapped, streamed through pinned buffers)."""
        self._check(self.lib.kcna_upload_lshkit(self.h, path.encode()))
        import struct
        with open(path, "rb") as f:
            _, _, d = struct.unpack("<III", f.read(12))
        self.n, self.d = (os.path.getsize(path) - 12) // (4 * d), d


def version() -> str:
    return load_library().kcna_version().decode()
