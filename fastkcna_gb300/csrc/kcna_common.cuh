// kcna_common.cuh - shared device helpers of the GB300 FastKCNA build library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kcna.h"

#define KCNA_WARP 32
#define KCNA_FULL 0xFFFFFFFFu
#define KCNA_NONE 0xFFFFFFFFu
#define KCNA_EMPTY_KEY 0xFFFFFFFFFFFFFFFFull
#define KCNA_EMPTY_KEY_NOFLAGS 0xFFFFFFFFFFFFFFFCull

// ---------------------------------------------------------------------------
// Pool entries are 64-bit keys ordered by (distance, id):
//   bits 63..32  IEEE bits of the FP32 squared distance (>= 0, so the bits are
//                monotonic in the value)
//   bits 31..2   node id (ids < 2^30)
//   bit 1        isnew: entry new relative to the previous prune loop
//   bit 0        flag: entry not yet used by a join / not yet pushed by P2K
// This replaces the 12-byte AoS Neighbor (src/neighbor.h:25-43); pid is not
// kept because every prune is a full prune.  Sorting keys as unsigned
// integers sorts by distance then id; a duplicate id has the same distance and
// sits next to its twin, so deduplication compares key >> 2.
// ---------------------------------------------------------------------------
#define KCNA_FLAG_NEW 1ull
#define KCNA_FLAG_ISNEW 2ull
#ifndef KCNA_MAX_ID
#define KCNA_MAX_ID ((1u << 30) - 1)
#endif

__device__ __forceinline__ uint64_t kcna_key(float dist, uint32_t id, uint32_t flags) {
    return ((uint64_t)__float_as_uint(dist) << 32) | ((uint64_t)id << 2) | (uint64_t)flags;
}
__device__ __forceinline__ float kcna_key_dist(uint64_t k) { return __uint_as_float((uint32_t)(k >> 32)); }
__host__ __device__ __forceinline__ uint32_t kcna_key_id(uint64_t k) { return (uint32_t)(k & 0xFFFFFFFFull) >> 2; }
__host__ __device__ __forceinline__ uint32_t kcna_key_flags(uint64_t k) { return (uint32_t)(k & 3ull); }
__host__ __device__ __forceinline__ uint64_t kcna_key_noflags(uint64_t k) { return k & ~3ull; }

// Candidate buffers: slot s (s = node * CB + position) holds the candidate's
// key in word 2 s and its joiner (the node whose join emitted it; low 32 bits)
// in word 2 s + 1, so one 16-byte store writes both.
__device__ __forceinline__ void kcna_cand_put(uint64_t *cand, uint64_t slot, uint64_t key, uint32_t joiner) {
    *reinterpret_cast<ulonglong2 *>(cand + 2 * slot) = make_ulonglong2(key, (unsigned long long)joiner);
}
__device__ __forceinline__ uint32_t kcna_cand_joiner(const uint64_t *cand, uint64_t slot) {
    return (uint32_t)cand[2 * slot + 1];
}

// ---------------------------------------------------------------------------
// Canonical FP32 squared L2 distance: one fused multiply-add chain over the
// dimensions in order, acc = fma(x_k - y_k, x_k - y_k, acc).  Every kernel that
// produces a stored or compared distance uses exactly this chain, so a pair
// gets the same bits wherever it is evaluated (the reference relies on this
// symmetry for its duplicate check, src/kgraph.cpp:261-298).  Rows are padded
// with zeros to a multiple of 4 floats; a zero term leaves acc unchanged.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float kcna_fma_step(float acc, float x, float y) {
    float t = __fsub_rn(x, y);
    return __fmaf_rn(t, t, acc);
}
__device__ __forceinline__ float kcna_acc4(float acc, float4 a, float4 b) {
    acc = kcna_fma_step(acc, a.x, b.x);
    acc = kcna_fma_step(acc, a.y, b.y);
    acc = kcna_fma_step(acc, a.z, b.z);
    acc = kcna_fma_step(acc, a.w, b.w);
    return acc;
}
// a, b 16-byte aligned, ld a multiple of 4
__device__ __forceinline__ float kcna_l2(const float *__restrict__ a, const float *__restrict__ b, int ld) {
    float acc = 0.f;
    const float4 *a4 = reinterpret_cast<const float4 *>(a);
    const float4 *b4 = reinterpret_cast<const float4 *>(b);
#pragma unroll 4
    for (int k = 0; k < (ld >> 2); ++k) acc = kcna_acc4(acc, a4[k], b4[k]);
    return acc;
}
// streaming read of a global row through the read-only path
__device__ __forceinline__ float kcna_l2_ldg(const float *__restrict__ a, const float *__restrict__ b, int ld) {
    float acc = 0.f;
    const float4 *a4 = reinterpret_cast<const float4 *>(a);
    const float4 *b4 = reinterpret_cast<const float4 *>(b);
#pragma unroll 4
    for (int k = 0; k < (ld >> 2); ++k) acc = kcna_acc4(acc, __ldg(a4 + k), __ldg(b4 + k));
    return acc;
}

// ---------------------------------------------------------------------------
// Row storage.  RowsF32 reads the FP32 rows; RowsB16 reads a BF16 copy, used
// only when every value of the data is exactly representable in BF16 (checked
// when the build starts), so both give the same floats and hence the same
// canonical distances with half the bytes.  ld4(r, k4) returns floats
// 4*k4 .. 4*k4+3 of row r.
// ---------------------------------------------------------------------------
struct RowsF32 {
    const float *p;
    int ld;
    __device__ __forceinline__ float4 ld4(uint64_t r, int k4) const {
        return __ldg(reinterpret_cast<const float4 *>(p + r * (uint64_t)ld) + k4);
    }
};
struct RowsB16 {
    const uint16_t *p;
    int ld;
    __device__ __forceinline__ float4 ld4(uint64_t r, int k4) const {
        const uint2 u = __ldg(reinterpret_cast<const uint2 *>(p + r * (uint64_t)ld) + k4);
        return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u), __uint_as_float(u.y << 16),
                           __uint_as_float(u.y & 0xFFFF0000u));
    }
};
// canonical distance between rows a and b of R
template <class R>
__device__ __forceinline__ float rows_l2(const R &rows, uint64_t a, uint64_t b) {
    float acc = 0.f;
    const int nv = rows.ld >> 2;
    for (int k0 = 0; k0 < nv; k0 += 8) { // eight loads of each row in flight
        float4 x[8], y[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const bool in = k0 + u < nv;
            x[u] = in ? rows.ld4(a, k0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
            y[u] = in ? rows.ld4(b, k0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (k0 + u < nv) acc = kcna_acc4(acc, x[u], y[u]);
    }
    return acc;
}

// ---------------------------------------------------------------------------
// Counter-based RNG (splitmix64) so that random draws depend only on
// (seed, stream, index) and not on thread scheduling.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t kcna_mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__host__ __device__ __forceinline__ uint32_t kcna_rand32(uint64_t seed, uint64_t stream, uint64_t i) {
    return (uint32_t)(kcna_mix64(seed * 0x100000001B3ull ^ kcna_mix64(stream * 0xD6E8FEB86659FD93ull + i)) >> 16);
}

// ---------------------------------------------------------------------------
// Device error word: kernels never trap; on an impossible condition they set a
// code (first writer wins) and skip the access.  The host reads it after each
// phase and turns it into KCNA_E_CUDA / KCNA_E_TIMEOUT.
// ---------------------------------------------------------------------------
enum {
    KCNA_DERR_NONE = 0,
    KCNA_DERR_BOUNDS = 1,   // an index fell outside its buffer
    KCNA_DERR_SPIN = 2,     // a bounded wait gave up
    KCNA_DERR_DEGREE = 3,   // a graph row ran out of slots
    KCNA_DERR_TIES = 4,     // more rows tie at the k-th distance than the selection holds
};
__device__ __forceinline__ void kcna_set_err(int *err, int code) {
    if (err) atomicCAS(err, 0, code);
}

// warp helpers
__device__ __forceinline__ int kcna_lane() { return threadIdx.x & 31; }
template <typename T>
__device__ __forceinline__ T kcna_warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(KCNA_FULL, v, o);
    return v;
}
__device__ __forceinline__ unsigned kcna_lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

static inline unsigned kcna_div_up(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }
