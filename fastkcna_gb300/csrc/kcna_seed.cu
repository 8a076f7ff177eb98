// kcna_seed.cu - learned seeding of NN-descent (no counterpart in the reference).
//
// The reference starts NN-descent from S random pool entries per node
// (src/kgraph.cpp:1001-1044).  This file replaces that start, when
// kcna_params.learned_seed is set, with pools drawn from learned codes:
//   1. a random subsample (up to 100,000 rows) gets a short GPU NN-descent;
//      its pools give (anchor, neighbour) pairs;
//   2. an MLP encoder x -> GELU(W1 x + b1) -> W2 . + b2 -> L2-normalise
//      (D -> 256 -> 64) is trained with the triplet loss
//      max(0, |f(a)-f(p)|^2 - |f(a)-f(n)|^2 + margin), Adam, on the tcgen05 BF16
//      GEMM (kcna_tc.cu) with FP32 master weights; every elementwise forward and
//      backward step below is a hand-written kernel;
//   3. every row is encoded; 16 tables each hash the 64-d code to 16 sign bits
//      of a random projection and counting-sort the rows by that bucket;
//   4. each node's initial pool is the exact FP32 distance-sorted union of its
//      +-w neighbours in the T sorted orders (self and duplicates dropped),
//      flagged new, after which NN-descent proceeds from its update step.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <random>
#include <vector>

#include "kcna_internal.h"
#include "kcna_sort.cuh"

namespace {

constexpr int H1 = 256, H2 = 64;
constexpr int SEED_TABLES = 16, SEED_BITS = 16, SEED_WIN = 32; // 16 tables x (2 x 32) = 1024 candidates per node
constexpr int SEED_CAND = SEED_TABLES * 2 * SEED_WIN;

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// Z1 = H + b1 (kept for the backward), G = GELU(Z1)
__global__ void bias_gelu_kernel(float *__restrict__ H, const float *__restrict__ b, float *__restrict__ G,
                                 int64_t rows, int cols) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * cols) return;
    const float z = H[t] + b[t % cols];
    H[t] = z;
    G[t] = gelu(z);
}

// Z2 = H + b2, nrm = |Z2|, Y = Z2 / nrm; one warp per row of 64
__global__ void bias_norm_kernel(const float *__restrict__ H, const float *__restrict__ b, float *__restrict__ Y,
                                 float *__restrict__ nrm, int64_t rows) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (r >= rows) return;
    const float z0 = H[r * H2 + lane] + b[lane], z1 = H[r * H2 + 32 + lane] + b[32 + lane];
    const float s = kcna_warp_sum(z0 * z0 + z1 * z1);
    const float n = fmaxf(sqrtf(s), 1e-12f);
    Y[r * H2 + lane] = z0 / n;
    Y[r * H2 + 32 + lane] = z1 / n;
    if (lane == 0) nrm[r] = n;
}

// Triplet loss over rows [a | p | n] of Y (B each); dY for all 3B rows; loss sum -> *loss
__global__ void triplet_kernel(const float *__restrict__ Y, int B, float margin, float *__restrict__ dY,
                               float *__restrict__ loss) {
    const int b = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = kcna_lane();
    if (b >= B) return;
    const float *ya = Y + (int64_t)b * H2, *yp = Y + (int64_t)(B + b) * H2, *yn = Y + (int64_t)(2 * B + b) * H2;
    float a0 = ya[lane], a1 = ya[lane + 32], p0 = yp[lane], p1 = yp[lane + 32], n0 = yn[lane], n1 = yn[lane + 32];
    const float dap = kcna_warp_sum((a0 - p0) * (a0 - p0) + (a1 - p1) * (a1 - p1));
    const float dan = kcna_warp_sum((a0 - n0) * (a0 - n0) + (a1 - n1) * (a1 - n1));
    const float l = dap - dan + margin;
    const float s = l > 0.f ? 2.f / B : 0.f;
    dY[(int64_t)b * H2 + lane] = s * (n0 - p0);
    dY[(int64_t)b * H2 + 32 + lane] = s * (n1 - p1);
    dY[(int64_t)(B + b) * H2 + lane] = s * (p0 - a0);
    dY[(int64_t)(B + b) * H2 + 32 + lane] = s * (p1 - a1);
    dY[(int64_t)(2 * B + b) * H2 + lane] = s * (a0 - n0);
    dY[(int64_t)(2 * B + b) * H2 + 32 + lane] = s * (a1 - n1);
    if (lane == 0 && l > 0.f) atomicAdd(loss, l / B);
}

// dZ2 = (dY - Y (Y . dY)) / nrm, in place on dY; one warp per row
__global__ void norm_bwd_kernel(const float *__restrict__ Y, const float *__restrict__ nrm, float *__restrict__ dY,
                                int64_t rows) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (r >= rows) return;
    const float y0 = Y[r * H2 + lane], y1 = Y[r * H2 + 32 + lane];
    const float g0 = dY[r * H2 + lane], g1 = dY[r * H2 + 32 + lane];
    const float dot = kcna_warp_sum(y0 * g0 + y1 * g1);
    const float n = nrm[r];
    dY[r * H2 + lane] = (g0 - y0 * dot) / n;
    dY[r * H2 + 32 + lane] = (g1 - y1 * dot) / n;
}

// dZ1 = dG * GELU'(Z1), in place on dG
__global__ void gelu_bwd_kernel(const float *__restrict__ Z, float *__restrict__ dG, int64_t n) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dG[t] *= gelu_grad(Z[t]);
}

// column sums of an (rows x cols) matrix in two deterministic passes: block
// (column group of 32, chunk of CS_ROWS rows) -> partial[chunk][col], then the
// chunks summed in order
constexpr int CS_ROWS = 256;
__global__ void colsum_partial_kernel(const float *__restrict__ M, int64_t rows, int cols,
                                      float *__restrict__ partial) {
    __shared__ float s[8][33];
    const int c = blockIdx.x * 32 + (threadIdx.x & 31), ry = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.y * CS_ROWS, r1 = min(rows, r0 + CS_ROWS);
    float acc = 0.f;
    if (c < cols)
        for (int64_t r = r0 + ry; r < r1; r += 8) acc += M[r * cols + c];
    s[ry][threadIdx.x & 31] = acc;
    __syncthreads();
    if (ry == 0 && c < cols) {
        float t = 0.f;
        for (int i = 0; i < 8; ++i) t += s[i][threadIdx.x];
        partial[(int64_t)blockIdx.y * cols + c] = t;
    }
}
__global__ void colsum_final_kernel(const float *__restrict__ partial, int nchunk, int cols, float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float t = 0.f;
    for (int k = 0; k < nchunk; ++k) t += partial[(int64_t)k * cols + c];
    out[c] = t;
}

__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int64_t n, float lr, float b1, float b2, float c1, float c2) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gi = g[t];
    const float mi = b1 * m[t] + (1.f - b1) * gi, vi = b2 * v[t] + (1.f - b2) * gi * gi;
    m[t] = mi;
    v[t] = vi;
    w[t] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

// batch rows [a | p | n] gathered from the subsample rows
__global__ void gather_triplets_kernel(const float *__restrict__ Xs, int ld, const uint32_t *__restrict__ trip,
                                       int B, float *__restrict__ Xb) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per = ld / 4;
    if (t >= (int64_t)3 * B * per) return;
    const int64_t r = t / per, c = t % per;
    const uint32_t src = trip[r];
    reinterpret_cast<float4 *>(Xb)[r * per + c] = reinterpret_cast<const float4 *>(Xs + (int64_t)src * ld)[c];
}

// triplets: anchor random, positive a random entry of the anchor's first kp pool entries, negative random
__global__ void make_triplets_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                     uint32_t cap, uint32_t ns, int kp, int B, uint64_t seed, uint32_t step,
                                     uint32_t *__restrict__ trip) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint32_t a = kcna_rand32(seed, step, 3ull * b) % ns;
    const uint32_t cnt = min(pool_cnt[a], (uint32_t)kp);
    uint32_t p = a;
    if (cnt > 0) p = kcna_key_id(pool[(uint64_t)a * cap + kcna_rand32(seed, step, 3ull * b + 1) % cnt]);
    if (p >= ns) p = a;
    const uint32_t n = kcna_rand32(seed, step, 3ull * b + 2) % ns;
    trip[b] = a;
    trip[B + b] = p;
    trip[2 * B + b] = n;
}

// 16 sign bits of the code against SEED_TABLES random projections
__global__ void hash_kernel(const float *__restrict__ Y, int64_t rows, const float *__restrict__ P,
                            uint32_t *__restrict__ bucket) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (r >= rows) return;
    const float y0 = Y[r * H2 + lane], y1 = Y[r * H2 + 32 + lane];
    for (int t = 0; t < SEED_TABLES; ++t) {
        uint32_t bits = 0;
        for (int j = 0; j < SEED_BITS; ++j) {
            const float *pj = P + ((int64_t)t * SEED_BITS + j) * H2;
            const float dot = kcna_warp_sum(y0 * pj[lane] + y1 * pj[lane + 32]);
            bits |= (dot >= 0.f ? 1u : 0u) << j;
        }
        if (lane == 0) bucket[(int64_t)t * rows + r] = bits;
    }
}

__global__ void bucket_count_kernel(const uint32_t *__restrict__ bucket, int64_t rows, uint32_t *__restrict__ hist) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * SEED_TABLES) return;
    const int64_t tab = t / rows;
    atomicAdd(hist + tab * (1 << SEED_BITS) + bucket[t], 1u);
}

__global__ void bucket_scatter_kernel(const uint32_t *__restrict__ bucket, int64_t rows,
                                      const uint64_t *__restrict__ off, uint32_t *__restrict__ cursor,
                                      uint32_t *__restrict__ order, uint32_t *__restrict__ rank) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * SEED_TABLES) return;
    const int64_t tab = t / rows, r = t % rows;
    const int64_t bi = tab * (1 << SEED_BITS) + bucket[t];
    const uint64_t pos = off[bi] + atomicAdd(cursor + bi, 1u) - (uint64_t)tab * rows;
    order[tab * rows + pos] = (uint32_t)r;
    rank[tab * rows + r] = (uint32_t)pos;
}

// Initial pool of node i, for rows too wide for the banded kernels below:
// sorted union of its +-SEED_WIN neighbours in every table order, with
// canonical distances (the node's row staged in shared
// memory; candidate rows read through R, the BF16 copy when it is exact).
template <class R>
__global__ void __launch_bounds__(128) seed_pools_kernel(R rows, uint32_t N, const uint32_t *__restrict__ order,
                                                         const uint32_t *__restrict__ rank, uint32_t cap,
                                                         uint32_t limit, uint64_t *__restrict__ pool,
                                                         uint32_t *__restrict__ pool_cnt,
                                                         unsigned long long *comps) {
    __shared__ uint64_t s_k[4][SEED_CAND];
    extern __shared__ __align__(16) float s_row[]; // 4 warps x ld
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    const uint32_t i = blockIdx.x * 4 + w;
    if (i >= N) return;
    const int nv = rows.ld >> 2;
    float4 *own = reinterpret_cast<float4 *>(s_row) + (size_t)w * nv;
    for (int k = lane; k < nv; k += 32) own[k] = rows.ld4(i, k);
    uint64_t *sk = s_k[w];
    for (int e = lane; e < SEED_CAND; e += 32) {
        const int tab = e / (2 * SEED_WIN), off = e % (2 * SEED_WIN);
        const int64_t pos = (int64_t)rank[(int64_t)tab * N + i] + (off < SEED_WIN ? off - SEED_WIN : off - SEED_WIN + 1);
        uint32_t id = KCNA_NONE;
        if (pos >= 0 && pos < (int64_t)N) id = order[(int64_t)tab * N + pos];
        sk[e] = (id == i || id >= N) ? KCNA_EMPTY_KEY : (uint64_t)id;
    }
    kcna_warp_bitonic(sk, SEED_CAND);
    // unique ids -> exact distances
    uint64_t keys[SEED_CAND / 32];
    unsigned long long cc = 0;
#pragma unroll
    for (int h = 0; h < SEED_CAND / 32; ++h) {
        const int e = h * 32 + lane;
        const uint64_t v = sk[e];
        const bool ok = v != KCNA_EMPTY_KEY && (e == 0 || sk[e - 1] != v);
        keys[h] = KCNA_EMPTY_KEY;
        if (ok) {
            ++cc;
            const uint32_t id = (uint32_t)v;
            float acc = 0.f;
            for (int k0 = 0; k0 < nv; k0 += 8) { // eight loads in flight
                float4 y[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) y[u] = k0 + u < nv ? rows.ld4(id, k0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (k0 + u < nv) acc = kcna_acc4(acc, y[u], own[k0 + u]);
            }
            keys[h] = kcna_key(acc, id, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
        }
    }
    __syncwarp();
#pragma unroll
    for (int h = 0; h < SEED_CAND / 32; ++h) sk[h * 32 + lane] = keys[h];
    kcna_warp_bitonic(sk, SEED_CAND);
    uint32_t cnt = 0;
    for (int e = 0; e < SEED_CAND; e += 32) cnt += __popc(__ballot_sync(KCNA_FULL, sk[e + lane] != KCNA_EMPTY_KEY));
    cnt = min(cnt, limit);
    uint64_t *pr = pool + (uint64_t)i * cap;
    for (uint32_t e = lane; e < cap; e += 32) pr[e] = e < cnt ? sk[e] : KCNA_EMPTY_KEY;
    cc = kcna_warp_sum(cc);
    if (lane == 0) {
        pool_cnt[i] = cnt;
        if (cc) atomicAdd(comps, cc);
    }
}

// Initial pools, step 1 (one launch, grid row tab for table tab): in the order
// of table tab, every position p meets
// positions p+1 .. p+SEED_WIN; each pair's canonical distance goes to both
// nodes' fixed candidate slots (node a's slot tab*2W + W + delta-1 holds the
// delta-th node after it, slot tab*2W + delta-1 the delta-th node before it).
// A warp stages the rows of its 32 positions and the SEED_WIN after them in
// shared memory as they are stored (BF16 or FP32; row pitch padded by 8 or 16
// bytes so that the lanes' reads fall in distinct banks), so each row is read
// from memory about twice per table instead of once per candidate; each lane
// keeps SEED_WIN running sums and reads its own row once per 4 dimensions.
constexpr int BAND_WARPS = 4, BAND_ROWS = 32 + SEED_WIN;

template <class R> struct BandStage;
template <> struct BandStage<RowsF32> {
    static constexpr int ELT = 4;
    __device__ static float4 get(const unsigned char *row, int k) {
        return reinterpret_cast<const float4 *>(row)[k];
    }
    __device__ static void put(unsigned char *row, int k, const float *src) {
        reinterpret_cast<float4 *>(row)[k] = __ldg(reinterpret_cast<const float4 *>(src) + k);
    }
};
template <> struct BandStage<RowsB16> {
    static constexpr int ELT = 2;
    __device__ static float4 get(const unsigned char *row, int k) {
        const uint2 u = reinterpret_cast<const uint2 *>(row)[k];
        return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u), __uint_as_float(u.y << 16),
                           __uint_as_float(u.y & 0xFFFF0000u));
    }
    __device__ static void put(unsigned char *row, int k, const uint16_t *src) {
        reinterpret_cast<uint2 *>(row)[k] = __ldg(reinterpret_cast<const uint2 *>(src) + k);
    }
};
__host__ __device__ constexpr int band_pitch(int ld, int elt) { return ld * elt + 4 * elt; } // bytes

template <class R>
__global__ void __launch_bounds__(BAND_WARPS * 32) seed_band_kernel(R rows, uint32_t N,
                                                                    const uint32_t *__restrict__ orders,
                                                                    uint64_t *__restrict__ slots, uint32_t stride,
                                                                    unsigned long long *comps) {
    using B = BandStage<R>;
    const int tab = (int)blockIdx.y; // one grid row per table
    const uint32_t *__restrict__ ord = orders + (size_t)tab * N;
    extern __shared__ __align__(16) unsigned char s_band[]; // BAND_WARPS x BAND_ROWS x pitch
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    const int nv = rows.ld >> 2, pitch = band_pitch(rows.ld, B::ELT);
    unsigned char *sr = s_band + (size_t)w * BAND_ROWS * pitch;
    const uint64_t p0 = ((uint64_t)blockIdx.x * BAND_WARPS + w) * 32;
    if (p0 >= N) return;
    const int nr = (int)min((uint64_t)BAND_ROWS, N - p0);
    for (int e = lane; e < nr * nv; e += 32) {
        const int r = e / nv, k = e - r * nv;
        B::put(sr + (size_t)r * pitch, k, rows.p + (uint64_t)ord[p0 + r] * rows.ld);
    }
    __syncwarp();
    const uint64_t p = p0 + lane;
    unsigned long long cc = 0;
    if (p < N) {
        const unsigned char *ra = sr + (size_t)lane * pitch;
        float acc[SEED_WIN];
#pragma unroll
        for (int d = 0; d < SEED_WIN; ++d) acc[d] = 0.f;
        for (int k = 0; k < nv; ++k) { // the canonical chain of every pair, dimension by dimension
            const float4 x = B::get(ra, k);
#pragma unroll
            for (int d = 0; d < SEED_WIN; ++d)
                if (lane + d + 1 < nr) acc[d] = kcna_acc4(acc[d], x, B::get(ra + (size_t)(d + 1) * pitch, k));
        }
        const uint32_t a = ord[p];
        const uint32_t fl = (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW);
#pragma unroll
        for (int d = 0; d < SEED_WIN; ++d) {
            if (lane + d + 1 >= nr) break;
            ++cc;
            const uint32_t b = ord[p + d + 1];
            slots[(uint64_t)a * stride + tab * 2 * SEED_WIN + SEED_WIN + d] = kcna_key(acc[d], b, fl);
            slots[(uint64_t)b * stride + tab * 2 * SEED_WIN + d] = kcna_key(acc[d], a, fl);
        }
    }
    cc = kcna_warp_sum(cc);
    if (lane == 0 && cc) atomicAdd(comps, cc);
}

// Initial pools, step 2: node i's slots sorted by (distance, id); the same id
// from several tables gives the same key, so repeats are adjacent and dropped;
// the nearest `limit` distinct entries become the pool.  Warp per node, the
// 1024 slots held in registers (32 per lane, slot 32 r + lane in k[r]) and
// sorted by a bitonic network: strides below 32 exchange across lanes by
// shuffles, larger strides between a lane's own registers.
static_assert(SEED_CAND == 1024, "the collect sort holds 32 keys per lane");

__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, int m) {
    const uint32_t lo = __shfl_xor_sync(KCNA_FULL, (uint32_t)v, m);
    const uint32_t hi = __shfl_xor_sync(KCNA_FULL, (uint32_t)(v >> 32), m);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t shfl_idx64(uint64_t v, int src) {
    const uint32_t lo = __shfl_sync(KCNA_FULL, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(KCNA_FULL, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t shfl_up64(uint64_t v, int d) {
    const uint32_t lo = __shfl_up_sync(KCNA_FULL, (uint32_t)v, d);
    const uint32_t hi = __shfl_up_sync(KCNA_FULL, (uint32_t)(v >> 32), d);
    return ((uint64_t)hi << 32) | lo;
}

// Ascending bitonic sort of the 1024 keys k[r] (key index 32 r + lane).
__device__ __forceinline__ void warp_sort1024(uint64_t (&k)[32], int lane) {
#pragma unroll
    for (int size = 2; size <= 1024; size <<= 1) {
#pragma unroll
        for (int j = size >> 1; j > 0; j >>= 1) {
            if (j >= 32) { // partner in this lane's register r ^ (j / 32)
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    if (r & jr) continue;
                    const bool asc = ((r * 32) & size) == 0;
                    const uint64_t x = k[r], y = k[r | jr];
                    const bool sw = asc ? x > y : x < y;
                    k[r] = sw ? y : x;
                    k[r | jr] = sw ? x : y;
                }
            } else { // partner in lane ^ j, same register
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    const bool asc = (((r * 32) | lane) & size) == 0;
                    const uint64_t x = k[r], y = shfl_xor64(x, j);
                    const bool keep_min = ((lane & j) == 0) == asc;
                    k[r] = keep_min ? (y < x ? y : x) : (y > x ? y : x);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(128) seed_collect_kernel(const uint64_t *__restrict__ slots, uint32_t stride,
                                                           uint32_t N, uint32_t cap, uint32_t limit,
                                                           uint64_t *__restrict__ pool,
                                                           uint32_t *__restrict__ pool_cnt) {
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    const uint32_t i = blockIdx.x * 4 + w;
    if (i >= N) return;
    const uint64_t *src = slots + (uint64_t)i * stride;
    uint64_t k[32];
#pragma unroll
    for (int r = 0; r < 32; ++r) k[r] = src[32 * r + lane];
    warp_sort1024(k, lane);
    uint64_t *pr = pool + (uint64_t)i * cap;
    uint32_t cnt = 0;
    uint64_t carry = KCNA_EMPTY_KEY;
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        const uint64_t v = k[r];
        uint64_t prev = shfl_up64(v, 1);
        if (lane == 0) prev = carry;
        carry = shfl_idx64(v, 31);
        const bool ok = v != KCNA_EMPTY_KEY && (r + lane == 0 || (prev >> 2) != (v >> 2));
        const unsigned m = __ballot_sync(KCNA_FULL, ok);
        const uint32_t pos = cnt + __popc(m & kcna_lanemask_lt());
        if (ok && pos < limit) pr[pos] = v;
        cnt += __popc(m);
    }
    const uint32_t keep = min(cnt, limit);
    for (uint32_t e = keep + lane; e < cap; e += 32) pr[e] = KCNA_EMPTY_KEY;
    if (lane == 0) pool_cnt[i] = keep;
}

__global__ void fill_u32_kernel(uint32_t *p, uint32_t v, uint64_t n) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}

struct Dev {
    kcna_ctx *c;
    std::vector<void *> bufs;
    ~Dev() {
        for (void *b : bufs) kcna_release(c, b);
    }
    template <typename T>
    kcna_status get(T **p, size_t n, const char *what) {
        *p = nullptr;
        kcna_status s = kcna_alloc(c, p, n, what);
        if (s == KCNA_OK) bufs.push_back(*p);
        return s;
    }
};

kcna_status launch_ok(kcna_ctx *c, const char *what, int n = 1) {
    c->launches += n;
    return kcna_cuda_check(c, cudaGetLastError(), what);
}

} // namespace

// One forward + backward pass of the encoder on 3B batch rows Xb (device,
// row pitch ld): loss, gradients.  Work buffers in `ws` (see below).
struct EncoderWork {
    float *Z1, *G, *H2, *Y, *nrm, *dY, *dG, *loss;
    float *part; // column-sum partials: ceil(rows / CS_ROWS) x H1
};
inline size_t colsum_parts(int64_t rows) { return (size_t)((rows + CS_ROWS - 1) / CS_ROWS) * H1; }
static void colsum(cudaStream_t s, const float *M, int64_t rows, int cols, float *part, float *out) {
    const int nchunk = (int)((rows + CS_ROWS - 1) / CS_ROWS);
    colsum_partial_kernel<<<dim3(kcna_div_up(cols, 32), nchunk), 256, 0, s>>>(M, rows, cols, part);
    colsum_final_kernel<<<kcna_div_up(cols, 256), 256, 0, s>>>(part, nchunk, cols, out);
}

static kcna_status encoder_fwd_bwd(kcna_ctx *c, const float *Xb, int ld, int B, const float *W1, const float *b1,
                                   const float *W2, const float *b2, float margin, EncoderWork &w, float *dW1,
                                   float *db1, float *dW2, float *db2) {
    cudaStream_t s = c->stream;
    const int64_t R = 3LL * B;
    KCNA_TRY(kcna_tc_gemm(s, Xb, ld, 1, 0, W1, ld, 1, 0, w.Z1, H1, (int)R, H1, ld, 0.f, c->d_err));
    bias_gelu_kernel<<<kcna_div_up(R * H1, 256), 256, 0, s>>>(w.Z1, b1, w.G, R, H1);
    KCNA_TRY(launch_ok(c, "bias_gelu", 2));
    KCNA_TRY(kcna_tc_gemm(s, w.G, H1, 1, 0, W2, H1, 1, 0, w.H2, H2, (int)R, H2, H1, 0.f, c->d_err));
    bias_norm_kernel<<<kcna_div_up(R * 32, 256), 256, 0, s>>>(w.H2, b2, w.Y, w.nrm, R);
    KCNA_TRY(launch_ok(c, "bias_norm", 2));
    cudaMemsetAsync(w.loss, 0, 4, s);
    triplet_kernel<<<kcna_div_up((int64_t)B * 32, 256), 256, 0, s>>>(w.Y, B, margin, w.dY, w.loss);
    norm_bwd_kernel<<<kcna_div_up(R * 32, 256), 256, 0, s>>>(w.Y, w.nrm, w.dY, R);
    KCNA_TRY(launch_ok(c, "triplet", 2));
    colsum(s, w.dY, R, H2, w.part, db2);
    // dW2 = dZ2^T G ; dG = dZ2 W2
    KCNA_TRY(kcna_tc_gemm(s, w.dY, H2, 1, 1, w.G, H1, 1, 1, dW2, H1, H2, H1, (int)R, 0.f, c->d_err));
    KCNA_TRY(kcna_tc_gemm(s, w.dY, H2, 1, 0, W2, H1, 1, 1, w.dG, H1, (int)R, H1, H2, 0.f, c->d_err));
    gelu_bwd_kernel<<<kcna_div_up(R * H1, 256), 256, 0, s>>>(w.Z1, w.dG, R * H1);
    colsum(s, w.dG, R, H1, w.part, db1);
    KCNA_TRY(launch_ok(c, "gelu_bwd", 6));
    // dW1 = dZ1^T Xb
    KCNA_TRY(kcna_tc_gemm(s, w.dG, H1, 1, 1, Xb, ld, 1, 1, dW1, ld, H1, ld, (int)R, 0.f, c->d_err));
    c->launches += 1;
    return KCNA_OK;
}

static void init_weights(std::vector<float> &W1, std::vector<float> &W2, int d, int ld, uint32_t seed) {
    std::mt19937 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    W1.assign((size_t)H1 * ld, 0.f);
    W2.assign((size_t)H2 * H1, 0.f);
    const float s1 = 1.f / std::sqrt((float)d), s2 = 1.f / std::sqrt((float)H1);
    for (int o = 0; o < H1; ++o)
        for (int i = 0; i < d; ++i) W1[(size_t)o * ld + i] = nd(rng) * s1;
    for (auto &v : W2) v = nd(rng) * s2;
}

// Learned initial pools for all c->n rows (pools must be allocated with cap).
kcna_status kcna_seed_learned(kcna_ctx *c, const kcna_params *p, kcna_stats *st) {
    const double t_start = kcna_now();
    const uint32_t N = c->n, ld = c->ld;
    cudaStream_t s = c->stream;
    Dev dev{c, {}};
    // --- 1. input scale: rows are divided by their global RMS so the encoder sees O(1) values
    // --- subsample and its NN-descent (a separate context on the same device)
    const uint32_t ns = std::min<uint32_t>(N, 100000);
    std::vector<uint32_t> sub(N);
    for (uint32_t i = 0; i < N; ++i) sub[i] = i;
    std::mt19937 rng(p->seed ^ 0x5EEDu);
    for (uint32_t i = 0; i < ns; ++i) std::swap(sub[i], sub[i + rng() % (N - i)]);
    uint32_t *d_sub = nullptr;
    float *Xs = nullptr;
    KCNA_TRY(dev.get(&d_sub, ns, "subsample ids"));
    KCNA_TRY(dev.get(&Xs, (size_t)ns * ld, "subsample rows"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(d_sub, sub.data(), (size_t)ns * 4, cudaMemcpyHostToDevice, s), "h2d"));
    KCNA_TRY(kcna_gather_rows(c, d_sub, ns, Xs));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(s), "subsample sync"));
    if (!c->seed_sub && kcna_create(&c->seed_sub, c->device) != KCNA_OK) {
        c->seed_sub = nullptr;
        return kcna_fail(c, KCNA_E_CUDA, "seed: no sub-context");
    }
    kcna_ctx *sc = c->seed_sub;
    if (kcna_upload_device(sc, Xs, ns, ld, (uint64_t)ld * 4) != KCNA_OK)
        return kcna_fail(c, KCNA_E_CUDA, std::string("seed: ") + kcna_last_error(sc));
    kcna_params sp;
    kcna_params_default(&sp);
    sp.K = sp.L = 32;
    sp.S = 10;
    sp.R = 32;
    sp.iterations = 4;
    sp.controls = 10;
    sp.search_L = sp.search_K = 32;
    sp.recall = 2.f; // run the iterations
    sp.delta = 0.f;
    sp.seed = p->seed + 17;
    sp.screen = p->screen; // Gram-exact tiles give the FP32 join's pools bit for bit
    kcna_stats sst;
    const uint64_t sub_launches0 = sc->launches;
    if (kcna_nndescent(sc, &sp, &sst) != KCNA_OK)
        return kcna_fail(c, KCNA_E_CUDA, std::string("seed subsample: ") + kcna_last_error(sc));
    c->launches += sc->launches - sub_launches0;
    // --- 2. encoder training
    const int B = 2048, steps = 64, kp = 10;
    const float margin = 0.3f, lr = 2e-3f;
    std::vector<float> hW1, hW2;
    init_weights(hW1, hW2, (int)c->d, (int)ld, p->seed + 101);
    float *W1, *b1, *W2, *b2, *dW1, *db1, *dW2, *db2, *mom, *vel;
    const size_t nW1 = (size_t)H1 * ld, nW2 = (size_t)H2 * H1, nparam = nW1 + H1 + nW2 + H2;
    float *params = nullptr, *grads = nullptr;
    KCNA_TRY(dev.get(&params, nparam, "encoder"));
    KCNA_TRY(dev.get(&grads, nparam, "encoder grads"));
    KCNA_TRY(dev.get(&mom, nparam, "adam m"));
    KCNA_TRY(dev.get(&vel, nparam, "adam v"));
    W1 = params;
    b1 = W1 + nW1;
    W2 = b1 + H1;
    b2 = W2 + nW2;
    dW1 = grads;
    db1 = dW1 + nW1;
    dW2 = db1 + H1;
    db2 = dW2 + nW2;
    cudaMemsetAsync(params, 0, nparam * 4, s);
    cudaMemsetAsync(mom, 0, nparam * 4, s);
    cudaMemsetAsync(vel, 0, nparam * 4, s);
    cudaMemcpyAsync(W1, hW1.data(), nW1 * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(W2, hW2.data(), nW2 * 4, cudaMemcpyHostToDevice, s);
    // rows scaled to unit RMS: the encoder's first layer absorbs the data range
    {
        std::vector<float> probe((size_t)std::min<uint32_t>(ns, 1024) * ld);
        cudaMemcpyAsync(probe.data(), Xs, probe.size() * 4, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        double ss = 0;
        for (float v : probe) ss += (double)v * v;
        const float rms = (float)std::sqrt(ss / std::max<size_t>(1, probe.size() / ld * c->d));
        const float inv = rms > 0 ? 1.f / rms : 1.f;
        for (auto &v : hW1) v *= inv; // scale folded into W1 instead of the data
        cudaMemcpyAsync(W1, hW1.data(), nW1 * 4, cudaMemcpyHostToDevice, s);
        c->stats = st; // for the record
        st->seed_input_scale = inv;
    }
    uint32_t *trip;
    float *Xb;
    EncoderWork w;
    const int64_t R = 3LL * B;
    KCNA_TRY(dev.get(&trip, (size_t)R, "triplets"));
    KCNA_TRY(dev.get(&Xb, (size_t)R * ld, "batch rows"));
    KCNA_TRY(dev.get(&w.Z1, (size_t)R * H1, "Z1"));
    KCNA_TRY(dev.get(&w.G, (size_t)R * H1, "G"));
    KCNA_TRY(dev.get(&w.H2, (size_t)R * H2, "H2"));
    KCNA_TRY(dev.get(&w.Y, (size_t)R * H2, "Y"));
    KCNA_TRY(dev.get(&w.nrm, (size_t)R, "nrm"));
    KCNA_TRY(dev.get(&w.dY, (size_t)R * H2, "dY"));
    KCNA_TRY(dev.get(&w.dG, (size_t)R * H1, "dG"));
    KCNA_TRY(dev.get(&w.loss, 1, "loss"));
    KCNA_TRY(dev.get(&w.part, colsum_parts(R), "column sums"));
    float first_loss = -1.f, last_loss = 0.f;
    for (int it = 0; it < steps; ++it) {
        make_triplets_kernel<<<kcna_div_up(B, 256), 256, 0, s>>>(sc->pool, sc->pool_cnt, sc->cap, ns, kp, B,
                                                                 p->seed + 7, (uint32_t)it, trip);
        gather_triplets_kernel<<<kcna_div_up(R * (ld / 4), 256), 256, 0, s>>>(Xs, (int)ld, trip, B, Xb);
        KCNA_TRY(launch_ok(c, "triplets", 2));
        KCNA_TRY(encoder_fwd_bwd(c, Xb, (int)ld, B, W1, b1, W2, b2, margin, w, dW1, db1, dW2, db2));
        const float c1 = 1.f - std::pow(0.9f, (float)(it + 1)), c2 = 1.f - std::pow(0.999f, (float)(it + 1));
        adam_kernel<<<kcna_div_up(nparam, 256), 256, 0, s>>>(params, grads, mom, vel, (int64_t)nparam, lr, 0.9f,
                                                             0.999f, c1, c2);
        KCNA_TRY(launch_ok(c, "adam"));
        if (it == 0 || it == steps - 1) {
            float h = 0.f;
            cudaMemcpyAsync(&h, w.loss, 4, cudaMemcpyDeviceToHost, s);
            KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(s), "train sync"));
            if (it == 0) first_loss = h;
            last_loss = h;
        }
    }
    st->seed_loss_first = first_loss;
    st->seed_loss_last = last_loss;
    const double t_train = kcna_now();
    // --- 3. encode all rows (chunks), hash into the tables
    const int64_t chunk = 262144;
    float *cz = nullptr, *cg = nullptr, *ch = nullptr, *Y = nullptr, *cn = nullptr;
    KCNA_TRY(dev.get(&cz, (size_t)chunk * H1, "encode Z1"));
    KCNA_TRY(dev.get(&cg, (size_t)chunk * H1, "encode G"));
    KCNA_TRY(dev.get(&ch, (size_t)chunk * H2, "encode H2"));
    KCNA_TRY(dev.get(&cn, (size_t)chunk, "encode nrm"));
    KCNA_TRY(dev.get(&Y, (size_t)N * H2, "codes"));
    for (int64_t r0 = 0; r0 < N; r0 += chunk) {
        const int64_t m = std::min<int64_t>(chunk, N - r0);
        KCNA_TRY(kcna_tc_gemm(s, c->X + r0 * ld, ld, 1, 0, W1, ld, 1, 0, cz, H1, (int)m, H1, ld, 0.f, c->d_err));
        bias_gelu_kernel<<<kcna_div_up(m * H1, 256), 256, 0, s>>>(cz, b1, cg, m, H1);
        KCNA_TRY(kcna_tc_gemm(s, cg, H1, 1, 0, W2, H1, 1, 0, ch, H2, (int)m, H2, H1, 0.f, c->d_err));
        bias_norm_kernel<<<kcna_div_up(m * 32, 256), 256, 0, s>>>(ch, b2, Y + r0 * H2, cn, m);
        KCNA_TRY(launch_ok(c, "encode", 4));
    }
    std::vector<float> hP((size_t)SEED_TABLES * SEED_BITS * H2);
    {
        std::normal_distribution<float> nd(0.f, 1.f);
        std::mt19937 prng(p->seed + 4242);
        for (auto &v : hP) v = nd(prng);
    }
    float *P = nullptr;
    uint32_t *bucket = nullptr, *hist = nullptr, *cursor = nullptr, *order = nullptr, *rank = nullptr;
    uint64_t *off = nullptr;
    const uint64_t nb = (uint64_t)SEED_TABLES << SEED_BITS;
    KCNA_TRY(dev.get(&P, hP.size(), "projections"));
    KCNA_TRY(dev.get(&bucket, (size_t)SEED_TABLES * N, "buckets"));
    KCNA_TRY(dev.get(&hist, nb, "bucket counts"));
    KCNA_TRY(dev.get(&cursor, nb, "bucket cursors"));
    KCNA_TRY(dev.get(&off, nb + 1, "bucket offsets"));
    KCNA_TRY(dev.get(&order, (size_t)SEED_TABLES * N, "orders"));
    KCNA_TRY(dev.get(&rank, (size_t)SEED_TABLES * N, "ranks"));
    cudaMemcpyAsync(P, hP.data(), hP.size() * 4, cudaMemcpyHostToDevice, s);
    hash_kernel<<<kcna_div_up((uint64_t)N * 32, 256), 256, 0, s>>>(Y, N, P, bucket);
    cudaMemsetAsync(hist, 0, nb * 4, s);
    cudaMemsetAsync(cursor, 0, nb * 4, s);
    bucket_count_kernel<<<kcna_div_up((uint64_t)N * SEED_TABLES, 256), 256, 0, s>>>(bucket, N, hist);
    KCNA_TRY(launch_ok(c, "hash", 2));
    KCNA_TRY(kcna_exclusive_scan_u32(c, hist, nb, off, nullptr));
    bucket_scatter_kernel<<<kcna_div_up((uint64_t)N * SEED_TABLES, 256), 256, 0, s>>>(bucket, N, off, cursor, order,
                                                                                     rank);
    KCNA_TRY(launch_ok(c, "bucket scatter"));
    // --- 4. initial pools
    const uint32_t limit = std::min(p->L, c->cap);
    cudaMemsetAsync(c->counters + 30, 0, 8, s);
    const size_t band_smem = (size_t)BAND_WARPS * BAND_ROWS * band_pitch((int)ld, c->bf16_exact ? 2 : 4);
    if (band_smem <= 200 * 1024) { // banded: each pair once, rows read in table order
        uint64_t *slots = c->cand;
        uint32_t stride = c->CB;
        if (c->CB < (uint32_t)SEED_CAND) {
            KCNA_TRY(dev.get(&slots, (size_t)N * SEED_CAND, "seed slots"));
            stride = SEED_CAND;
        }
        KCNA_TRY(kcna_cuda_check(c, cudaMemset2DAsync(slots, (size_t)stride * 8, 0xFF, (size_t)SEED_CAND * 8, N, s),
                                 "memset"));
        auto band = [&](auto rows) -> kcna_status {
            KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(seed_band_kernel<decltype(rows)>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                             (int)band_smem),
                                     "seed band smem attr"));
            seed_band_kernel<<<dim3(kcna_div_up(N, 32 * BAND_WARPS), SEED_TABLES), BAND_WARPS * 32, band_smem, s>>>(
                rows, N, order, slots, stride, c->counters + 30);
            return launch_ok(c, "seed band");
        };
        if (c->bf16_exact)
            KCNA_TRY(band(RowsB16{c->Xh, (int)ld}));
        else
            KCNA_TRY(band(RowsF32{c->X, (int)ld}));
        seed_collect_kernel<<<kcna_div_up(N, 4), 128, 0, s>>>(slots, stride, N, c->cap, limit, c->pool, c->pool_cnt);
    } else {
        const size_t srow = (size_t)4 * ld * 4;
        if (c->bf16_exact)
            seed_pools_kernel<<<kcna_div_up(N, 4), 128, srow, s>>>(RowsB16{c->Xh, (int)ld}, N, order, rank, c->cap,
                                                                   limit, c->pool, c->pool_cnt, c->counters + 30);
        else
            seed_pools_kernel<<<kcna_div_up(N, 4), 128, srow, s>>>(RowsF32{c->X, (int)ld}, N, order, rank, c->cap,
                                                                   limit, c->pool, c->pool_cnt, c->counters + 30);
    }
    KCNA_TRY(launch_ok(c, "seed pools"));
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, c->counters + 30, 8, cudaMemcpyDeviceToHost, s);
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(s), "seed sync"));
    st->seed_comps = h;
    st->seed_train_ms = (t_train - t_start) * 1000.0;
    st->seed_total_ms = (kcna_now() - t_start) * 1000.0;
    return kcna_check_device_err(c, "learned seed");
}

// M = S and found = 1 for every node, so that the first update samples the
// S nearest pool entries as the new list (the reference's init sets M = S).
kcna_status kcna_seed_finish(kcna_ctx *c, const kcna_params *p) {
    fill_u32_kernel<<<kcna_div_up(c->n, 256), 256, 0, c->stream>>>(c->M, p->S, c->n);
    cudaMemsetAsync(c->found, 1, c->n, c->stream);
    KCNA_TRY(launch_ok(c, "seed finish"));
    c->has_pools = true;
    return kcna_pools_set_radius(c, p->L);
}

extern "C" kcna_status kcna_encoder_grads(kcna_ctx *c, const float *rows, uint32_t n_rows, uint32_t d, const float *W1,
                                          const float *b1, const float *W2, const float *b2, float margin, float *loss,
                                          float *dW1, float *db1, float *dW2, float *db2) {
    if (!c) return KCNA_E_ARG;
    if (!rows || !W1 || !b1 || !W2 || !b2 || !loss || !dW1 || !db1 || !dW2 || !db2 || d == 0 || n_rows == 0 ||
        n_rows % 3)
        return kcna_fail(c, KCNA_E_ARG, "encoder_grads: bad argument (rows must be 3B)");
    KCNA_TRY(kcna_cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice"));
    const int ld = (int)((d + 3) & ~3u), B = (int)(n_rows / 3);
    const int64_t R = n_rows;
    cudaStream_t s = c->stream;
    Dev dev{c, {}};
    float *Xb, *pW1, *pb1, *pW2, *pb2, *gW1, *gb1, *gW2, *gb2;
    EncoderWork w;
    KCNA_TRY(dev.get(&Xb, (size_t)R * ld, "rows"));
    KCNA_TRY(dev.get(&pW1, (size_t)H1 * ld, "W1"));
    KCNA_TRY(dev.get(&pb1, H1, "b1"));
    KCNA_TRY(dev.get(&pW2, (size_t)H2 * H1, "W2"));
    KCNA_TRY(dev.get(&pb2, H2, "b2"));
    KCNA_TRY(dev.get(&gW1, (size_t)H1 * ld, "dW1"));
    KCNA_TRY(dev.get(&gb1, H1, "db1"));
    KCNA_TRY(dev.get(&gW2, (size_t)H2 * H1, "dW2"));
    KCNA_TRY(dev.get(&gb2, H2, "db2"));
    KCNA_TRY(dev.get(&w.Z1, (size_t)R * H1, "Z1"));
    KCNA_TRY(dev.get(&w.G, (size_t)R * H1, "G"));
    KCNA_TRY(dev.get(&w.H2, (size_t)R * H2, "H2"));
    KCNA_TRY(dev.get(&w.Y, (size_t)R * H2, "Y"));
    KCNA_TRY(dev.get(&w.nrm, (size_t)R, "nrm"));
    KCNA_TRY(dev.get(&w.dY, (size_t)R * H2, "dY"));
    KCNA_TRY(dev.get(&w.dG, (size_t)R * H1, "dG"));
    KCNA_TRY(dev.get(&w.loss, 1, "loss"));
    KCNA_TRY(dev.get(&w.part, colsum_parts(R), "column sums"));
    cudaMemsetAsync(Xb, 0, (size_t)R * ld * 4, s);
    cudaMemsetAsync(pW1, 0, (size_t)H1 * ld * 4, s);
    cudaMemcpy2DAsync(Xb, (size_t)ld * 4, rows, (size_t)d * 4, (size_t)d * 4, R, cudaMemcpyHostToDevice, s);
    cudaMemcpy2DAsync(pW1, (size_t)ld * 4, W1, (size_t)d * 4, (size_t)d * 4, H1, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(pb1, b1, H1 * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(pW2, W2, (size_t)H2 * H1 * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(pb2, b2, H2 * 4, cudaMemcpyHostToDevice, s);
    KCNA_TRY(encoder_fwd_bwd(c, Xb, ld, B, pW1, pb1, pW2, pb2, margin, w, gW1, gb1, gW2, gb2));
    cudaMemcpyAsync(loss, w.loss, 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpy2DAsync(dW1, (size_t)d * 4, gW1, (size_t)ld * 4, (size_t)d * 4, H1, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(db1, gb1, H1 * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(dW2, gW2, (size_t)H2 * H1 * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(db2, gb2, H2 * 4, cudaMemcpyDeviceToHost, s);
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(s), "encoder_grads"));
    return kcna_check_device_err(c, "encoder_grads");
}
