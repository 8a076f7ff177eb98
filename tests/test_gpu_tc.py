"""tcgen05 BF16 GEMM (kcna_gemm_bf16) against an FP32 product of the same
BF16 values.  Integer-valued operands are exact in BF16 and their products
and sums stay below 2^24, so that case must match bit for bit."""
import ctypes as C

import numpy as np
import pytest

from fastkcna_gb300 import kcna

pytestmark = pytest.mark.gpu


def gemm(A, B, a_trans=False, b_trans=False, M=None, N=None, K=None):
    import torch

    lib = kcna.load_library()
    f = lib.kcna_gemm_bf16
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p,
                  C.c_int64, C.c_int, C.c_int, C.c_int, C.c_void_p]
    out = torch.empty((M, N), dtype=torch.float32, device=A.device)
    rc = f(A.data_ptr(), A.stride(0), int(A.dtype == torch.float32), int(a_trans), B.data_ptr(), B.stride(0),
           int(B.dtype == torch.float32), int(b_trans), out.data_ptr(), N, M, N, K,
           torch.cuda.current_stream().cuda_stream)
    assert rc == 0, rc
    return out


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 128), (200, 100, 96), (77, 33, 16), (1000, 256, 256)])
def test_gemm_bf16_matches_fp32_product(M, N, K):
    import torch

    g = torch.Generator(device="cpu").manual_seed(M * 7 + N)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    ref = A.float() @ B.float().T
    got = gemm(A, B, M=M, N=N, K=K)
    torch.testing.assert_close(got, ref, rtol=1e-4, atol=1e-4)


def test_gemm_integer_data_exact():
    import torch

    g = torch.Generator(device="cpu").manual_seed(3)
    A = torch.randint(0, 256, (256, 128), generator=g).float().cuda()  # fp32 storage, integers 0..255
    B = torch.randint(0, 256, (192, 128), generator=g).float().cuda()
    got = gemm(A, B, M=256, N=192, K=128)
    ref = (A.double() @ B.double().T).float()
    assert torch.equal(got, ref)


def test_gemm_split_k_long_reduction():
    import torch

    g = torch.Generator(device="cpu").manual_seed(9)
    At = torch.randn(6144, 64, generator=g).cuda()   # stored K x M (fp32), the weight-gradient shape
    Bt = torch.randn(6144, 256, generator=g).cuda()  # stored K x N
    ref = At.to(torch.bfloat16).double().T @ Bt.to(torch.bfloat16).double()
    got = gemm(At, Bt, a_trans=True, b_trans=True, M=64, N=256, K=6144)
    torch.testing.assert_close(got.double(), ref, rtol=1e-3, atol=1e-2)


def test_gemm_transposed_operands():
    import torch

    g = torch.Generator(device="cpu").manual_seed(5)
    At = torch.randn(96, 150, generator=g).to(torch.bfloat16).cuda()  # stored K x M
    Bt = torch.randn(96, 70, generator=g).float().cuda()               # stored K x N, fp32
    ref = At.float().T @ Bt.to(torch.bfloat16).float()
    got = gemm(At, Bt, a_trans=True, b_trans=True, M=150, N=70, K=96)
    torch.testing.assert_close(got, ref, rtol=1e-4, atol=1e-4)
