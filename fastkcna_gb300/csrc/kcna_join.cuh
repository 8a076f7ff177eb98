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
    uint64_t *cand;     // key and joiner per slot (kcna_cand_put)
    uint32_t *cand_cnt;
    uint32_t CB;
    uint8_t *found;
    unsigned long long *counters; // [0] pairs evaluated, [5] rows gathered, [6] candidates emitted
    uint32_t capA, capB;          // list capacities in shared memory (forward + R)
    int *err;
};

// tcgen05 Gram-tile join over the BF16 rows (kcna_join_tc.cu); requires
// c->gram_exact (see kcna_internal.h).
kcna_status kcna_join_tc_launch(kcna_ctx *c, const JoinArgs &a);
// whether the lists of this build fit the Gram-tile join's shared memory
bool kcna_join_tc_fits(const JoinArgs &a);

namespace {

// Random stream of node `node`'s reverse subset in iteration `iter`
// (old = 0: reverse new list, 1: reverse old list).
__device__ __forceinline__ uint64_t join_reverse_stream(uint32_t iter, uint32_t node, uint32_t old) {
    return ((uint64_t)iter << 40) ^ ((uint64_t)node << 1) ^ (uint64_t)old;
}

// Copies the reverse list a join reads: its first min(cnt, R) entries (the
// random subset select_reverse_kernel left there).  The caller synchronises
// before the copy is read.
__device__ __forceinline__ uint32_t take_reverse(const uint32_t *src, uint32_t cnt, uint32_t R, uint32_t *dst) {
    const uint32_t m = min(cnt, R);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) dst[i] = src[i];
    return m;
}

} // namespace
