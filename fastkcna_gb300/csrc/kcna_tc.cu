// kcna_tc.cu - BF16 tensor-core GEMM on tcgen05 (sm_103a).
//
// C[M x N] (FP32, row-major) = A[M x K] * B[N x K]^T, operands read as FP32
// or BF16, optionally transposed, converted to BF16 while they are staged
// into 128B-swizzled shared memory tiles; one thread issues the tcgen05.mma
// instructions (M = 128, N = 64, K = 16), the accumulator lives in TMEM and is
// read back with tcgen05.ld.  Used by the learned-seed encoder (forward and
// backward products) and exported as kcna_gemm_bf16 for tests and callers.
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int TM = 128, TN = 64, TK = 64; // tile: 128 rows of A, 64 rows of B, 64 K-elements per stage

struct Operand {
    const void *p;
    int64_t ld;  // elements between consecutive rows of the stored matrix
    int fp32;    // 1: FP32 storage, 0: BF16 storage
    int trans;   // 1: element (r, k) stored at p[k * ld + r]
};

__device__ __forceinline__ float load_elem(const Operand &o, int64_t r, int64_t k) {
    const int64_t idx = o.trans ? k * o.ld + r : r * o.ld + k;
    return o.fp32 ? __ldg(reinterpret_cast<const float *>(o.p) + idx)
                  : __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(o.p)[idx]);
}

// rows [r0, r0+nrows) x K-elements [k0, k0+64) of o, zero outside [0,rows) x [0,K)
__device__ void stage(uint8_t *tile, const Operand &o, int64_t r0, int nrows, int64_t rows, int64_t k0, int64_t K) {
    for (int idx = threadIdx.x; idx < nrows * 8; idx += blockDim.x) {
        const int r = idx >> 3, c = idx & 7;
        float f[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int64_t k = k0 + c * 8 + e;
            f[e] = (r0 + r < rows && k < K) ? load_elem(o, r0 + r, k) : 0.f;
        }
        *reinterpret_cast<uint4 *>(tile + sw128_off(r, c)) = pack8_bf16(f);
    }
}

// gridDim.z > 1 splits K: slice z covers [z*kslice, (z+1)*kslice) and adds its
// partial product into C with atomicAdd (C cleared by the caller).
__global__ void __launch_bounds__(128) tc_gemm_kernel(Operand A, Operand B, float *__restrict__ C, int64_t ldc,
                                                      int M, int N, int K, float beta, int64_t kslice, int *err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t s_tmem;
    const uint32_t base_s = (smem_u32(smem_raw) + 1023u) & ~1023u; // 1024-byte aligned for the swizzle
    uint8_t *base = smem_raw + (base_s - smem_u32(smem_raw));
    uint8_t *sA = base;           // 128 rows x 128 bytes
    uint8_t *sB = base + TM * 128; // 64 rows x 128 bytes
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = (int64_t)blockIdx.x * TM, n0 = (int64_t)blockIdx.y * TN;
    if (warp == 0) tmem_alloc(&s_tmem, TN);
    if (tid == 0) {
        mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t idesc = idesc_bf16(TM, TN);
    uint32_t phase = 0;
    bool ok = true;
    const int64_t kbeg = (int64_t)blockIdx.z * kslice, kend = min((int64_t)K, kbeg + kslice);
    for (int64_t k0 = kbeg; k0 < kend; k0 += TK) {
        stage(sA, A, m0, TM, M, k0, kend);
        stage(sB, B, n0, TN, N, k0, kend);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int kk = 0; kk < TK / 16; ++kk)
                mma_bf16(tmem, desc_sw128(base_s + kk * 32), desc_sw128(base_s + TM * 128 + kk * 32), idesc,
                         (k0 > kbeg || kk > 0) ? 1u : 0u);
            mma_commit(&mbar);
        }
        ok = mbar_wait(&mbar, phase) && ok; // the MMAs have read the tiles: they may be overwritten
        phase ^= 1u;
    }
    fence_after();
    const int64_t row = m0 + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < TN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (row < M) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int64_t col = n0 + c0 + i;
                if (col < N) {
                    float *dst = C + row * ldc + col;
                    if (gridDim.z > 1)
                        atomicAdd(dst, v[i]);
                    else
                        *dst = beta != 0.f ? v[i] + beta * *dst : v[i];
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, TN);
    if (!ok && tid == 0) kcna_set_err(err, KCNA_DERR_SPIN);
}

__device__ int g_tc_err; // error word of the exported GEMM

} // namespace

constexpr size_t TC_SMEM = (size_t)(TM + TN) * 128 + 1024;

kcna_status kcna_tc_gemm(cudaStream_t s, const void *A, int64_t lda, int a_fp32, int a_trans, const void *B,
                         int64_t ldb, int b_fp32, int b_trans, float *C, int64_t ldc, int M, int N, int K, float beta,
                         int *err) {
    if (M <= 0 || N <= 0 || K <= 0) return KCNA_E_ARG;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) !=
            cudaSuccess)
            return KCNA_E_CUDA;
        attr = true;
    }
    Operand a{A, lda, a_fp32, a_trans}, b{B, ldb, b_fp32, b_trans};
    dim3 grid((M + TM - 1) / TM, (N + TN - 1) / TN);
    // long reductions (K much larger than the output tile count) are split over K
    int64_t kslice = ((int64_t)K + TK - 1) / TK * TK;
    const int64_t tiles = (int64_t)grid.x * grid.y;
    if (tiles < 64 && K >= 1024) {
        const int64_t splits = std::min<int64_t>((K + 511) / 512, std::max<int64_t>(1, 256 / tiles));
        kslice = ((K + splits - 1) / splits + TK - 1) / TK * TK;
        grid.z = (unsigned)((K + kslice - 1) / kslice);
    }
    if (grid.z > 1) {
        if (beta != 0.f) return KCNA_E_ARG;
        if (cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, (size_t)M, s) != cudaSuccess) return KCNA_E_CUDA;
    }
    tc_gemm_kernel<<<grid, 128, TC_SMEM, s>>>(a, b, C, ldc, M, N, K, beta, kslice, err);
    return cudaGetLastError() == cudaSuccess ? KCNA_OK : KCNA_E_CUDA;
}

extern "C" kcna_status kcna_gemm_bf16(const void *A, int64_t lda, int a_fp32, int a_trans, const void *B, int64_t ldb,
                                      int b_fp32, int b_trans, float *C, int64_t ldc, int M, int N, int K,
                                      void *stream) {
    int *err = nullptr;
    if (cudaGetSymbolAddress((void **)&err, g_tc_err) != cudaSuccess) {
        (void)cudaGetLastError();
        return KCNA_E_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(err, 0, 4, s) != cudaSuccess) return KCNA_E_CUDA;
    kcna_status st = kcna_tc_gemm(s, A, lda, a_fp32, a_trans, B, ldb, b_fp32, b_trans, C, ldc, M, N, K, 0.f, err);
    if (st != KCNA_OK) return st;
    int h = 0;
    if (cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return KCNA_E_CUDA;
    return h ? KCNA_E_TIMEOUT : KCNA_OK;
}
