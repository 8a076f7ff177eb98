"""The allocation-free exact k-NN entry point (kcna_knn_queries_noalloc).

It exists for callers that cannot call cudaMalloc where they need neighbours
(a fixed-budget arena that owns all device memory, a plugin inside another
framework's allocator).  The test allocates the device buffers itself, as such
a caller would, calls the entry point through the C ABI twice in a row, and
compares each result with the ordinary entry point (kcna_knn_queries): ids and
distances must be identical, the same bit-exact bar as the other k-NN tests.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu


def _noalloc(lib, base, queries, k, stream, expect=0):
    import torch

    n, d = base.shape
    m = queries.shape[0]
    out_i = torch.empty((m, k), dtype=torch.int32, device=base.device)
    out_d = torch.empty((m, k), dtype=torch.float32, device=base.device)
    f = lib.kcna_knn_queries_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32,
                  C.c_void_p, C.c_void_p, C.c_void_p]
    rc = f(base.data_ptr(), n, d, base.stride(0) * 4, queries.data_ptr(), m, queries.stride(0) * 4, k,
           out_i.data_ptr(), out_d.data_ptr(), stream)
    assert rc == expect, rc
    return out_i.cpu().numpy().view(np.uint32), out_d.cpu().numpy()


def test_noalloc_matches_allocating_entry_point():
    import torch

    X = synth.base("c2", 20000)
    Q1 = synth.queries("c2", 300)  # > one scratch batch (209 rows of 20,000 distances)
    Q2 = synth.queries("c1", 40)
    X2 = synth.base("c1", 5000)
    lib = kcna.load_library()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    with kcna.Index(0) as ix:
        ix.upload(X)
        ref_i1, ref_d1 = ix.knn_queries(Q1, 100)
        ix.upload(X2)
        ref_i2, ref_d2 = ix.knn_queries(Q2, 64)
    b1, q1 = torch.from_numpy(X).to(dev), torch.from_numpy(Q1).to(dev)
    b2, q2 = torch.from_numpy(X2).to(dev), torch.from_numpy(Q2).to(dev)
    got_i1, got_d1 = _noalloc(lib, b1, q1, 100, stream)
    got_i2, got_d2 = _noalloc(lib, b2, q2, 64, stream)  # second call reuses the scratch
    assert np.array_equal(got_i1, ref_i1) and np.array_equal(got_d1, ref_d1)
    assert np.array_equal(got_i2, ref_i2) and np.array_equal(got_d2, ref_d2)


def test_noalloc_rejects_oversize():
    import torch

    lib = kcna.load_library()
    f = lib.kcna_knn_queries_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32,
                  C.c_void_p, C.c_void_p, C.c_void_p]
    dev = torch.device("cuda", 0)
    t = torch.zeros((8, 16), dtype=torch.float32, device=dev)
    # n beyond the 16 MiB scratch: rejected before any device work
    assert f(t.data_ptr(), 5_000_000, 16, 64, t.data_ptr(), 1, 64, 10, t.data_ptr(), t.data_ptr(), None) == 1
    assert f(t.data_ptr(), 8, 15, 64, t.data_ptr(), 1, 64, 4, t.data_ptr(), t.data_ptr(), None) == 1  # d % 4
    assert f(t.data_ptr(), 8, 16, 64, t.data_ptr(), 1, 64, 9, t.data_ptr(), t.data_ptr(), None) == 1  # k > n


def test_noalloc_tie_overflow_status_and_recovery():
    """More than 1024 base rows at the k-th distance is a property of the data:
    the call reports KCNA_E_LIMIT (7), and the next call, which clears the shared
    error word, succeeds with the same results as the allocating entry point."""
    import torch

    lib = kcna.load_library()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    X = np.ones((1100, 16), np.float32)  # 1,100 identical rows: every distance ties
    _noalloc(lib, torch.from_numpy(X).to(dev), torch.from_numpy(X[:2].copy()).to(dev), 4, stream, expect=7)
    Y = synth.base("c1", 3000)
    Yq = synth.queries("c1", 20)
    with kcna.Index(0) as ix:
        ix.upload(Y)
        ref_i, ref_d = ix.knn_queries(Yq, 8)
    got_i, got_d = _noalloc(lib, torch.from_numpy(Y).to(dev), torch.from_numpy(Yq).to(dev), 8, stream)
    assert np.array_equal(got_i, ref_i) and np.array_equal(got_d, ref_d)
