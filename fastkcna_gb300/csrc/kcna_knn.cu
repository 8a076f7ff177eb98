// kcna_knn.cu - exact k-NN (brute force) on the GPU.
//
// Replaces LinearSearch (src/kgraph.cpp:309-330, used by GenerateControl
// :363-387) and SearchOracle::search (:332-361): for each query, the k rows
// with the smallest squared L2 distance, ties broken by the lower id (the
// reference scans ids in order and inserts equal distances after existing
// ones, src/kgraph.cpp:227-260).  Two kernels:
//   1. a tiled distance kernel (32 queries x 128 rows per block, 4x4 register
//      micro-tiles, dimensions staged through shared memory in chunks of 32)
//      computing the canonical FMA-chain distance of every pair;
//   2. an exact selection kernel per query: three radix-histogram passes over
//      the distance bits find the k-th smallest distance T, then every row with
//      distance < T plus the lowest ids among rows with distance == T are kept
//      and sorted by (distance, id).
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_sort.cuh"

namespace {

constexpr int TQ = 32, TB = 128, KC = 32, KCP = KC + 4;

__global__ void __launch_bounds__(256) dist_tile_kernel(const float *__restrict__ Q, uint32_t m,
                                                        const float *__restrict__ X, uint32_t n, int ld,
                                                        const uint32_t *__restrict__ q_self, float *__restrict__ D,
                                                        uint64_t ldD) {
    __shared__ __align__(16) float Qs[TQ][KCP];
    __shared__ __align__(16) float Xs[TB][KCP];
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const uint32_t q0 = blockIdx.y * TQ;
    const uint64_t b0 = (uint64_t)blockIdx.x * TB;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

    for (int k0 = 0; k0 < ld; k0 += KC) {
        {   // Q chunk: 32 rows x 32 floats, one float4 per thread
            int r = tid >> 3, c = (tid & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q0 + r < m && k0 + c < ld) v = *reinterpret_cast<const float4 *>(Q + (uint64_t)(q0 + r) * ld + k0 + c);
            *reinterpret_cast<float4 *>(&Qs[r][c]) = v;
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) { // X chunk: 128 rows x 32 floats
            int idx = tid + s * 256;
            int r = idx >> 3, c = (idx & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (b0 + r < n && k0 + c < ld) v = __ldg(reinterpret_cast<const float4 *>(X + (b0 + r) * ld + k0 + c));
            *reinterpret_cast<float4 *>(&Xs[r][c]) = v;
        }
        __syncthreads();
        const int kend = min(KC, ld - k0);
        for (int k = 0; k < kend; k += 4) {
            float4 qa[4], xb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) qa[i] = *reinterpret_cast<const float4 *>(&Qs[ty + 8 * i][k]);
#pragma unroll
            for (int j = 0; j < 4; ++j) xb[j] = *reinterpret_cast<const float4 *>(&Xs[tx + 32 * j][k]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = kcna_acc4(acc[i][j], qa[i], xb[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uint32_t q = q0 + ty + 8 * i;
        if (q >= m) continue;
        uint32_t self = q_self ? q_self[q] : KCNA_NONE;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint64_t b = b0 + tx + 32 * j;
            if (b >= n) continue;
            D[(uint64_t)q * ldD + b] = (b == self) ? __uint_as_float(0x7F800000u) : acc[i][j];
        }
    }
}

constexpr int SEL_T = 512;
constexpr int SEL_BINS = 4096;
constexpr int SEL_MAXK = 1024;
constexpr int SEL_TIES = 1024;

// Finds the bin holding the want-th (0-based) element; returns bin and the
// number of elements in lower bins.  hist has nb bins (multiple of SEL_T).
__device__ void find_bin(const uint32_t *hist, int nb, uint32_t want, uint32_t *s_scan, int *out_bin,
                         uint32_t *out_before) {
    const int per = nb / SEL_T;
    uint32_t local = 0;
    for (int i = 0; i < per; ++i) local += hist[threadIdx.x * per + i];
    s_scan[threadIdx.x] = local;
    __syncthreads();
    // inclusive Hillis-Steele scan over SEL_T partial sums
    for (int off = 1; off < SEL_T; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? s_scan[threadIdx.x - off] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t incl = s_scan[threadIdx.x], excl = incl - local;
    if (want >= excl && want < incl) {
        uint32_t run = excl;
        for (int i = 0; i < per; ++i) {
            uint32_t h = hist[threadIdx.x * per + i];
            if (want < run + h) {
                *out_bin = threadIdx.x * per + i;
                *out_before = run;
                break;
            }
            run += h;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SEL_T) select_kernel(const float *__restrict__ D, uint64_t ldD, uint32_t n,
                                                       uint32_t k, uint32_t q_base, uint32_t *__restrict__ out_ids,
                                                       float *__restrict__ out_d, int *err) {
    __shared__ uint32_t hist[SEL_BINS];
    __shared__ uint32_t s_scan[SEL_T];
    __shared__ uint64_t s_out[SEL_MAXK];
    __shared__ uint64_t s_tie[SEL_TIES];
    __shared__ int s_bin;
    __shared__ uint32_t s_before, s_nout, s_ntie;
    const uint32_t *row = reinterpret_cast<const uint32_t *>(D + (uint64_t)blockIdx.x * ldD);
    uint32_t want = k - 1, prefix = 0;
    // three passes: bits 31..20, 19..8, 7..0
    const int shifts[3] = {20, 8, 0};
    const int widths[3] = {12, 12, 8};
    for (int pass = 0; pass < 3; ++pass) {
        const int sh = shifts[pass], nb = 1 << widths[pass];
        for (int i = threadIdx.x; i < SEL_BINS; i += SEL_T) hist[i] = 0;
        __syncthreads();
        const int hsh = sh + widths[pass];
        for (uint32_t j = threadIdx.x; j < n; j += SEL_T) {
            uint32_t v = row[j];
            if (pass == 0 || (v >> hsh) == prefix) atomicAdd(&hist[(v >> sh) & (nb - 1)], 1u);
        }
        __syncthreads();
        find_bin(hist, nb < SEL_T ? SEL_T : nb, want, s_scan, &s_bin, &s_before);
        prefix = (prefix << widths[pass]) | (uint32_t)s_bin;
        want -= s_before;
        __syncthreads();
    }
    const uint32_t T = prefix; // k-th smallest distance bits
    if (threadIdx.x == 0) {
        s_nout = 0;
        s_ntie = 0;
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < n; j += SEL_T) {
        uint32_t v = row[j];
        if (v < T) {
            uint32_t p = atomicAdd(&s_nout, 1u);
            if (p < SEL_MAXK) s_out[p] = ((uint64_t)v << 32) | j;
        } else if (v == T) {
            uint32_t p = atomicAdd(&s_ntie, 1u);
            if (p < SEL_TIES) s_tie[p] = ((uint64_t)v << 32) | j;
        }
    }
    __syncthreads();
    uint32_t nless = s_nout, ntie = s_ntie;
    if (ntie > SEL_TIES) kcna_set_err(err, KCNA_DERR_TIES);
    if (nless >= k) kcna_set_err(err, KCNA_DERR_BOUNDS);
    ntie = min(ntie, (uint32_t)SEL_TIES);
    nless = min(nless, k);
    int tp = kcna_pow2_ceil_d((int)ntie);
    for (int i = ntie + threadIdx.x; i < tp; i += SEL_T) s_tie[i] = KCNA_EMPTY_KEY;
    kcna_cta_bitonic(s_tie, tp);
    uint32_t need = k - nless;
    for (uint32_t i = threadIdx.x; i < need; i += SEL_T) s_out[nless + i] = i < ntie ? s_tie[i] : KCNA_EMPTY_KEY;
    int kp = kcna_pow2_ceil_d((int)k);
    for (int i = k + threadIdx.x; i < kp; i += SEL_T) s_out[i] = KCNA_EMPTY_KEY;
    kcna_cta_bitonic(s_out, kp);
    const uint64_t ob = (uint64_t)(q_base + blockIdx.x) * k;
    for (uint32_t i = threadIdx.x; i < k; i += SEL_T) {
        uint64_t key = s_out[i];
        out_ids[ob + i] = (uint32_t)key;
        out_d[ob + i] = __uint_as_float((uint32_t)(key >> 32));
    }
}

__global__ void gather_rows_kernel(const float *__restrict__ X, int ld, const uint32_t *__restrict__ ids, uint32_t m,
                                   uint32_t n, float *__restrict__ dst, int *err) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t total = (uint64_t)m * (ld / 4);
    if (t >= total) return;
    uint32_t r = (uint32_t)(t / (ld / 4)), c = (uint32_t)(t % (ld / 4));
    uint32_t id = ids[r];
    if (id >= n) {
        kcna_set_err(err, KCNA_DERR_BOUNDS);
        return;
    }
    reinterpret_cast<float4 *>(dst)[t] = reinterpret_cast<const float4 *>(X + (uint64_t)id * ld)[c];
}

} // namespace

kcna_status kcna_gather_rows(kcna_ctx *c, const uint32_t *d_ids, uint32_t m, float *dst) {
    uint64_t total = (uint64_t)m * (c->ld / 4);
    if (!total) return KCNA_OK;
    gather_rows_kernel<<<kcna_div_up(total, 256), 256, 0, c->stream>>>(c->X, c->ld, d_ids, m, c->n, dst, c->d_err);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "gather_rows");
}

kcna_status kcna_knn_device(kcna_ctx *c, const float *dQ, uint32_t m, const uint32_t *q_self, uint32_t k,
                            uint32_t *d_out_ids, float *d_out_d) {
    if (k == 0 || k > SEL_MAXK || k > c->n) return kcna_fail(c, KCNA_E_ARG, "knn: k must be in [1, min(1024, n)]");
    if (q_self && k >= c->n) return kcna_fail(c, KCNA_E_ARG, "knn: k must be < n when self is excluded");
    // distance rows for a batch of queries; batch bounded to ~1 GiB of scratch
    uint64_t row_bytes = (uint64_t)c->n * sizeof(float);
    uint32_t batch = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(m, (1ull << 30) / row_bytes));
    batch = std::max<uint32_t>(batch - batch % TQ, std::min<uint32_t>(batch, TQ));
    batch = std::min<uint32_t>(batch, 65535u * TQ); // grid.y limit of the distance tiles
    void *buf = nullptr;
    KCNA_TRY(kcna_scratch(c, (uint64_t)batch * row_bytes, &buf));
    float *D = (float *)buf;
    for (uint32_t q0 = 0; q0 < m; q0 += batch) {
        uint32_t mb = std::min(batch, m - q0);
        dim3 grid(kcna_div_up(c->n, TB), kcna_div_up(mb, TQ));
        dist_tile_kernel<<<grid, 256, 0, c->stream>>>(dQ + (uint64_t)q0 * c->ld, mb, c->X, c->n, (int)c->ld,
                                                      q_self ? q_self + q0 : nullptr, D, c->n);
        KCNA_LAUNCHED(c);
        select_kernel<<<mb, SEL_T, 0, c->stream>>>(D, c->n, c->n, k, q0, d_out_ids, d_out_d, c->d_err);
        KCNA_LAUNCHED(c);
        KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "knn kernels"));
    }
    return KCNA_OK;
}
