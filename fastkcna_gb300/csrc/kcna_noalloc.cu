// kcna_noalloc.cu - exact k-NN of device-resident queries that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they need nearest
// neighbours: code running under a fixed memory budget that owns every byte
// of the device through its own arena, plugins called from inside another
// framework's allocator-controlled region, or callers that must not take the
// driver's allocation lock on a latency-critical path.  For them this file
// offers kcna_knn_queries_noalloc: the caller passes the base rows, the
// queries and the outputs (all in device memory), and the only working memory
// is a fixed array in the library's own device image (g_scratch below, of
// KCNA_NOALLOC_SCRATCH_BYTES), which every GPU that loads the library holds
// until the process exits.
//
// Results are those of kcna_knn_queries: the canonical FMA-chain distance and
// ties broken by the lower row id.
#include <algorithm>
#include <mutex>

#include "kcna_common.cuh"
#include "kcna_sort.cuh"

namespace {

constexpr int TQ = 32, TB = 128, KC = 32, KCP = KC + 4;
constexpr int SEL_T = 512, SEL_BINS = 4096, SEL_MAXK = 1024, SEL_TIES = 1024;
constexpr size_t HEADER = 256; // error word lives in the first 256 bytes

// The scratch: a 256-byte header (error word) followed by distance rows.
static __device__ __align__(256) unsigned char g_scratch[KCNA_NOALLOC_SCRATCH_BYTES];

// Distances of a batch of queries to all base rows, canonical FMA chain.
// Strides are in floats; dims is a multiple of 4 (checked on the host).
__global__ void __launch_bounds__(256) na_dist_kernel(const float *__restrict__ Q, uint32_t m, uint64_t qs,
                                                      const float *__restrict__ X, uint32_t n, uint64_t xs, int dims,
                                                      float *__restrict__ D) {
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
    for (int k0 = 0; k0 < dims; k0 += KC) {
        {
            int r = tid >> 3, c = (tid & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q0 + r < m && k0 + c < dims) v = *reinterpret_cast<const float4 *>(Q + (uint64_t)(q0 + r) * qs + k0 + c);
            *reinterpret_cast<float4 *>(&Qs[r][c]) = v;
        }
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            int idx = tid + s * 256;
            int r = idx >> 3, c = (idx & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (b0 + r < n && k0 + c < dims) v = __ldg(reinterpret_cast<const float4 *>(X + (b0 + r) * xs + k0 + c));
            *reinterpret_cast<float4 *>(&Xs[r][c]) = v;
        }
        __syncthreads();
        const int kend = min(KC, dims - k0);
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
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint64_t b = b0 + tx + 32 * j;
            if (b < n) D[(uint64_t)q * n + b] = acc[i][j];
        }
    }
}

__device__ void na_find_bin(const uint32_t *hist, int nb, uint32_t want, uint32_t *s_scan, int *out_bin,
                            uint32_t *out_before) {
    const int per = nb / SEL_T;
    uint32_t local = 0;
    for (int i = 0; i < per; ++i) local += hist[threadIdx.x * per + i];
    s_scan[threadIdx.x] = local;
    __syncthreads();
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

// Exact k smallest (distance, id) of one distance row per block.
__global__ void __launch_bounds__(SEL_T) na_select_kernel(const float *__restrict__ D, uint32_t n, uint32_t k,
                                                          uint32_t *__restrict__ out_ids, float *__restrict__ out_d,
                                                          int *err) {
    __shared__ uint32_t hist[SEL_BINS];
    __shared__ uint32_t s_scan[SEL_T];
    __shared__ uint64_t s_out[SEL_MAXK];
    __shared__ uint64_t s_tie[SEL_TIES];
    __shared__ int s_bin;
    __shared__ uint32_t s_before, s_nout, s_ntie;
    const uint32_t *row = reinterpret_cast<const uint32_t *>(D + (uint64_t)blockIdx.x * n);
    uint32_t want = k - 1, prefix = 0;
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
        na_find_bin(hist, nb < SEL_T ? SEL_T : nb, want, s_scan, &s_bin, &s_before);
        prefix = (prefix << widths[pass]) | (uint32_t)s_bin;
        want -= s_before;
        __syncthreads();
    }
    const uint32_t T = prefix;
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
    if (threadIdx.x == 0 && ntie > SEL_TIES) atomicCAS(err, 0, KCNA_DERR_TIES);
    if (threadIdx.x == 0 && nless >= k) atomicCAS(err, 0, KCNA_DERR_BOUNDS);
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
    const uint64_t ob = (uint64_t)blockIdx.x * k;
    for (uint32_t i = threadIdx.x; i < k; i += SEL_T) {
        uint64_t key = s_out[i];
        out_ids[ob + i] = (uint32_t)key;
        out_d[ob + i] = __uint_as_float((uint32_t)(key >> 32));
    }
}

// Device address of g_scratch, looked up once per device.
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char *g_addr[MAX_DEVICES] = {};

kcna_status scratch_address(int dev, unsigned char **out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return KCNA_E_CUDA;
        }
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return KCNA_OK;
}

} // namespace

extern "C" kcna_status kcna_knn_queries_noalloc(const float *d_base, uint32_t n, uint32_t d,
                                                uint64_t base_stride_bytes, const float *d_queries, uint32_t m,
                                                uint64_t q_stride_bytes, uint32_t k, uint32_t *d_out_ids,
                                                float *d_out_dists, void *stream) {
    const size_t rows_bytes = KCNA_NOALLOC_SCRATCH_BYTES - HEADER;
    if (!d_base || !d_queries || !d_out_ids || !d_out_dists || m == 0) return KCNA_E_ARG;
    if (d == 0 || d % 4 || base_stride_bytes % 16 || q_stride_bytes % 16 || base_stride_bytes < (uint64_t)d * 4 ||
        q_stride_bytes < (uint64_t)d * 4 || ((uintptr_t)d_base & 15) || ((uintptr_t)d_queries & 15))
        return KCNA_E_ARG; // float4 loads: d a multiple of 4, 16-byte aligned rows
    if (k == 0 || k > SEL_MAXK || k > n) return KCNA_E_ARG;
    if ((uint64_t)n * sizeof(float) > rows_bytes) return KCNA_E_ARG; // one distance row must fit the scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        (void)cudaGetLastError();
        return KCNA_E_CUDA;
    }
    unsigned char *base = nullptr;
    kcna_status st = scratch_address(dev, &base);
    if (st != KCNA_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // a runtime error left pending on this host thread by earlier work is
    // reported, and left in place for its owner, rather than consumed here
    if (cudaPeekAtLastError() != cudaSuccess) return KCNA_E_CUDA;
    int *err = reinterpret_cast<int *>(base);
    float *D = reinterpret_cast<float *>(base + HEADER);
    // the scratch keeps the previous call's contents: the error word must start at zero
    if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) {
        (void)cudaGetLastError();
        return KCNA_E_CUDA;
    }
    // rows of distances that fit the scratch, and at most 65,535 query tiles
    // (the grid's y limit) per launch
    const uint32_t batch = (uint32_t)std::min<uint64_t>(rows_bytes / ((uint64_t)n * sizeof(float)), 65535ull * TQ);
    const uint64_t qs = q_stride_bytes / 4, xs = base_stride_bytes / 4;
    for (uint32_t q0 = 0; q0 < m; q0 += batch) {
        const uint32_t mb = m - q0 < batch ? m - q0 : batch;
        dim3 grid((n + TB - 1) / TB, (mb + TQ - 1) / TQ);
        na_dist_kernel<<<grid, 256, 0, s>>>(d_queries + (uint64_t)q0 * qs, mb, qs, d_base, n, xs, (int)d, D);
        na_select_kernel<<<mb, SEL_T, 0, s>>>(D, n, k, d_out_ids + (uint64_t)q0 * k, d_out_dists + (uint64_t)q0 * k,
                                              err);
        if (cudaPeekAtLastError() != cudaSuccess) {
            (void)cudaGetLastError(); // this call's own launch error
            return KCNA_E_CUDA;
        }
    }
    int h = 0;
    if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        (void)cudaGetLastError();
        return KCNA_E_CUDA;
    }
    if (h == KCNA_DERR_TIES) return KCNA_E_LIMIT; // more than 1024 rows tie at the k-th distance
    return h ? KCNA_E_CUDA : KCNA_OK;
}
