// kcna_join.cuh - arguments and list assembly shared by the two local-join
// kernels (FP32 register tiles in kcna_nnd.cu, tcgen05 Gram tiles in
// kcna_join_tc.cu).  Both draw the same random reverse subsets, so for equal
// distances they emit the same candidates.
#pragma once
#include "kcna_common.cuh"

struct kcna_ctx;

struct JoinArgs {
    const float *X;
    int ld;
    uint32_t N;
    uint32_t iter;
    uint64_t seed;
    uint32_t R, RB;
    const uint32_t *fwd_new, *fwd_new_cnt;
    uint32_t fwd_new_cap;
    const uint32_t *fwd_old, *fwd_old_cnt;
    uint32_t fwd_old_cap;
    const uint32_t *rnew, *rnew_cnt, *rold, *rold_cnt;
    const float *radius;
    uint64_t *cand;
    uint32_t *cand_cnt;
    uint32_t CB;
    uint8_t *found;
    unsigned long long *counters; // [0] pairs evaluated, [5] rows gathered, [6] candidates emitted
    uint32_t capA, capB;          // list capacities in shared memory (forward + RB)
    int *err;
};

// tcgen05 Gram-tile join over the BF16 rows (kcna_join_tc.cu); requires
// c->gram_exact (see kcna_internal.h).
kcna_status kcna_join_tc_launch(kcna_ctx *c, const JoinArgs &a);

namespace {

// Random stream of node `node`'s reverse subset in iteration `iter`
// (old = 0: reverse new list, 1: reverse old list).
__device__ __forceinline__ uint64_t join_reverse_stream(uint32_t iter, uint32_t node, uint32_t old) {
    return ((uint64_t)iter << 40) ^ ((uint64_t)node << 1) ^ (uint64_t)old;
}

// Copies up to R of cnt (capped at RB <= 4 * blockDim.x) reverse entries, a
// random subset when more (the reference shuffles rnn_* and keeps R,
// src/kgraph.cpp:1183-1201).  The entries are first put in ascending id order,
// so the subset depends only on the set of entries and not on the order in
// which concurrent writers appended them: a run is reproducible as long as no
// reverse list overflows RB.
__device__ void take_reverse(const uint32_t *src, uint32_t cnt, uint32_t RB, uint32_t R, uint64_t seed,
                             uint64_t stream, uint32_t *dst, uint32_t *s_n) {
    uint32_t m = min(cnt, RB);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    if (m > R) {
        constexpr int PER = 4;
        uint32_t v[PER], rk[PER];
#pragma unroll
        for (int e = 0; e < PER; ++e) {
            const uint32_t i = threadIdx.x + e * blockDim.x;
            v[e] = i < m ? dst[i] : 0u;
            rk[e] = 0u;
        }
#pragma unroll
        for (int e = 0; e < PER; ++e) { // rank = position in (id, index) order
            const uint32_t i = threadIdx.x + e * blockDim.x;
            if (e * blockDim.x >= m) break;
            if (i < m)
                for (uint32_t j = 0; j < m; ++j) {
                    const uint32_t w = dst[j];
                    rk[e] += (w < v[e] || (w == v[e] && j < i)) ? 1u : 0u;
                }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < PER; ++e)
            if (threadIdx.x + e * blockDim.x < m) dst[rk[e]] = v[e];
        __syncthreads();
        if (threadIdx.x == 0) { // partial Fisher-Yates
            for (uint32_t i = 0; i < R; ++i) {
                uint32_t j = i + kcna_rand32(seed, stream, i) % (m - i);
                uint32_t t = dst[i];
                dst[i] = dst[j];
                dst[j] = t;
            }
        }
        m = R;
    }
    if (threadIdx.x == 0) *s_n = m;
    __syncthreads();
}

} // namespace
