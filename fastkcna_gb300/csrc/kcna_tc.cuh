// kcna_tc.cuh - 5th-generation tensor core (tcgen05) building blocks for sm_103a.
//
// BF16 x BF16 -> FP32 products C = A * B^T with both operands K-major, issued
// by one thread per CTA with tcgen05.mma (M = 128, N = NT, K = 16 per
// instruction), the accumulator in tensor memory (TMEM), and read back with
// tcgen05.ld.  Operand tiles are staged by the CTA's threads into shared
// memory in the 128-byte swizzled K-major layout (8-row groups of 1024 bytes;
// the 16-byte chunk c of row r sits at chunk c ^ (r % 8)), so rows can be
// gathered, converted from FP32 and transposed while staging.
#pragma once
#include <cuda_bf16.h>

#include "kcna_common.cuh"

namespace kcna_tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);    // start address (16-byte units)
    d |= (uint64_t)1 << 16;                      // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;            // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                      // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                      // layout: 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: A and B BF16, D FP32, both K-major.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of the 16-byte chunk c (0..7) of row r in a swizzled tile.
__device__ __forceinline__ uint32_t sw128_off(uint32_t r, uint32_t c) {
    return (r >> 3) * 1024u + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4);
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// One warp: allocate ncols (power of two >= 32) TMEM columns; address -> *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Bounded wait on an mbarrier phase: mbarrier.try_wait suspends the thread
// in hardware (up to the time hint, a microsecond, per try) instead of
// polling, so waiting warps take no issue slots; after 64 tries each further
// try also sleeps, so the bound holds whatever the suspension; false when
// max_tries tries (a second or more) ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t max_tries = (1u << 20)) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < max_tries; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(1000u)
            : "memory");
        if (done) return true;
        if (i > 64) __nanosleep(256);
    }
    return false;
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane, without
// waiting: the registers are valid after tmem_wait_ld().
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
// Waits for this thread's outstanding tcgen05.ld; r (16 registers of one load)
// is tied to the wait so that no use of it is scheduled before.
__device__ __forceinline__ void tmem_wait_ld16(uint32_t *r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane, waited for.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    tmem_ld16_async(taddr, r);
    tmem_wait_ld16(r);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// mbarrier arrive (release, CTA scope) by this thread.
__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(mbar))
                 : "memory");
}
// Arrive on mbar once every cp.async this thread issued so far has landed
// (the arrival counts towards the barrier's expected count).
__device__ __forceinline__ void mbar_arrive_cp_async(uint64_t *mbar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}
// mbarrier arrive by this thread that also raises the barrier's expected
// transaction count by `bytes` (bulk copies then complete them).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(mbar)),
                 "r"(bytes)
                 : "memory");
}
// Bulk (TMA engine) copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) global -> shared, completing `bytes` transactions on mbar.
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}

// Named barrier over `count` threads (a multiple of 32), id 1..15.
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// 4-byte asynchronous copy global -> shared (through L1).
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}

// 16-byte asynchronous copy global -> shared (L2 only), and the wait for all
// of this thread's copies.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Packs 8 floats into 8 BF16 (round to nearest even) as one 16-byte chunk.
__device__ __forceinline__ uint4 pack8_bf16(const float *f) {
    uint4 o;
    __nv_bfloat162 t;
    t = __floats2bfloat162_rn(f[0], f[1]);
    o.x = *reinterpret_cast<uint32_t *>(&t);
    t = __floats2bfloat162_rn(f[2], f[3]);
    o.y = *reinterpret_cast<uint32_t *>(&t);
    t = __floats2bfloat162_rn(f[4], f[5]);
    o.z = *reinterpret_cast<uint32_t *>(&t);
    t = __floats2bfloat162_rn(f[6], f[7]);
    o.w = *reinterpret_cast<uint32_t *>(&t);
    return o;
}

} // namespace kcna_tc
