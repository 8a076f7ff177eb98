// kcna_prune_tc.cu - occlusion prune on tcgen05 Gram tiles.
//
// Same result as prune_kernel (kcna_graph.cu; reference nsg_sync_prune
// src/kgraph.cpp:1809-1851, taumg_sync_prune :2833-2876, alphapg_sync_prune
// :3157-3203): the candidates of node q are pool[first .. lim) in order; the
// first is kept; a later candidate p is dropped when an already kept t
// occludes it (RNG: d(t,p) < d(q,p); tau-MNG: d(t,p) < d(q,p) - 3 tau;
// alpha-PG: d(t,p) < d(q,p) and the angle test), and the scan stops at range
// kept.  Candidate-to-candidate distances come from Gram tiles on BF16 rows
// ((|x|^2 + |y|^2) - 2 <x, y>, FP32 accumulation in TMEM); the kernel runs
// only in Gram-exact mode (integer rows, squared norms below 2^23), where they
// equal the canonical FMA-chain distances, so the kept lists are identical.
//
// One node at a time per block (128 threads, thread = candidate row of the
// current chunk; several blocks per SM overlap).  Per chunk of 128
// candidates:
//   1. TMA tile::gather4 of the chunk's BF16 rows (128-byte swizzle);
//   2. Gram tile chunk x kept rows (kept so far, N <= 128): a candidate
//      occluded by an earlier kept one is dead;
//   3. Gram tile chunk x chunk: thread p builds the 128-bit mask of the
//      earlier chunk candidates that would occlude it;
//   4. one warp scans the chunk in order, a mask word at a time: p is kept
//      when alive and no kept chunk candidate is in its mask; the scan stops
//      at range;
//   5. the newly kept rows are copied into the kept tile for the next chunk.
// Waits are bounded; a wait that gives up sets the error word and ends the
// block after its products have finished.
#include <cuda.h>

#include <algorithm>

#include "kcna_internal.h"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int PT = 128;                     // threads = candidate rows per chunk
constexpr uint32_t KBB = 128;               // bytes of a row inside one 64-element K block
constexpr uint32_t CHUNK = PT * KBB * 2;    // 32 KiB of BF16 rows (d <= 128)
constexpr int KMAX = 128;                   // kept rows (range <= 128)
constexpr uint32_t KEPT = KMAX * KBB * 2;   // 32 KiB
constexpr uint32_t TCOLS = 128;             // TMEM columns: one 128-column accumulator

struct PruneTcArgs {
    uint32_t N, cap, W;
    const uint64_t *pool;
    const uint32_t *pool_cnt;
    const float *norms;
    int kind;
    float t3, thr;
    int range, maxc;
    uint32_t *g_ids;
    float *g_dist;
    uint32_t *g_deg;
    unsigned long long *comps;
    int *err;
};

__device__ __forceinline__ bool occl(int kind, float t3, float thr, float td, float djk, float pd) {
    if (kind == KCNA_TAUMNG) return djk < __fsub_rn(pd, t3);
    if (kind == KCNA_ALPHAPG) {
        const float num = __fdiv_rn(__fsub_rn(__fadd_rn(td, djk), pd), 2.0f);
        const float cs = __fdiv_rn(num, __fsqrt_rn(__fmul_rn(td, djk)));
        return djk < pd && cs < thr;
    }
    return djk < pd;
}

__global__ void __launch_bounds__(PT, 3) prune_tc_kernel(PruneTcArgs a, const __grid_constant__ CUtensorMap tmap,
                                                      int ldh) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t bar_rows, bar_mma;
    __shared__ uint32_t s_tmem;
    __shared__ uint32_t s_id[PT];
    __shared__ float s_pd[PT], s_nrm[PT];
    __shared__ __align__(16) uint32_t s_mask[PT][4]; // earlier chunk candidates that would occlude row p
    __shared__ uint32_t s_alive[4];
    __shared__ uint32_t k_id[KMAX];
    __shared__ float k_pd[KMAX], k_nrm[KMAX];
    __shared__ int s_nk, s_newk, s_kfrom[KMAX];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    const uint32_t tC = tiles_s, tK = tiles_s + CHUNK;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (ldh + 63) >> 6;
    const void *tm = &tmap;

    if (warp == 0) tmem_alloc(&s_tmem, TCOLS);
    if (tid == 0) {
        mbar_init(&bar_rows, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // K padding of the kept tile beyond ldh and its unused rows read as zero
    for (int i = tid; i < (int)((CHUNK + KEPT) / 16); i += PT) reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    uint32_t ph_rows = 0, ph_mma = 0;
    bool ok = true;
    unsigned long long cc = 0;

    for (uint32_t q = blockIdx.x; q < a.N && ok; q += gridDim.x) {
        const uint64_t *pr = a.pool + (uint64_t)q * a.cap;
        const int cnt = (int)a.pool_cnt[q];
        int first = 0;
        if (cnt > 0 && kcna_key_id(pr[0]) == q) first = 1;
        const int lim = max(min(cnt, a.maxc), first + 1);
        if (tid == 0) s_nk = 0;
        int nk = 0;
        if (first < cnt) {
            for (int c0 = first; c0 < lim && nk < a.range && ok; c0 += PT) {
                const int m = min(PT, lim - c0); // candidates of this chunk
                // metadata and rows of the chunk
                uint32_t id = 0xFFFFFFFFu;
                float pd = 0.f;
                if (tid < m) {
                    const uint64_t k = pr[c0 + tid];
                    id = kcna_key_id(k);
                    pd = kcna_key_dist(k);
                }
                const bool live = tid < m && id < a.N; // src/kgraph.cpp:1822, ids beyond the prefix are skipped
                s_id[tid] = tid < m ? id : 0u;
                s_pd[tid] = pd;
                s_nrm[tid] = live ? __ldg(a.norms + id) : __uint_as_float(0x7FC00000u);
                __syncthreads();
                if (tid == 0) mbar_arrive_expect_tx(&bar_rows, (uint32_t)((m + 3) / 4 * 4 * nkb) * KBB);
                __syncthreads();
                if (tid < 32) {
                    const int ng = (m + 3) >> 2;
                    for (int e = lane; e < ng * nkb; e += 32) {
                        const int g = nkb == 2 ? e >> 1 : e, kb = nkb == 2 ? e & 1 : 0;
                        const int r = 4 * g;
                        tma_gather4(tC + (uint32_t)kb * PT * KBB + (uint32_t)r * KBB, tm, 64 * kb, (int)s_id[r],
                                    (int)s_id[min(r + 1, m - 1)], (int)s_id[min(r + 2, m - 1)],
                                    (int)s_id[min(r + 3, m - 1)], &bar_rows);
                    }
                }
                ok = mbar_wait(&bar_rows, ph_rows) && ok;
                ph_rows ^= 1u;
                // 2. against the rows kept so far (columns 0..nk-1)
                bool alive = live;
                if (nk > 0) {
                    if (tid == 0) {
                        fence_after();
                        const uint32_t idesc = idesc_bf16(PT, (nk + 15) & ~15);
                        for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk)
                                mma_bf16(tmem, desc_sw128(tC + kb * PT * KBB + kk * 32),
                                         desc_sw128(tK + kb * KMAX * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
                        mma_commit(&bar_mma);
                    }
                    ok = mbar_wait(&bar_mma, ph_mma) && ok;
                    ph_mma ^= 1u;
                    fence_after();
                    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
                    for (int g = 0; g * 16 < nk; ++g) {
                        uint32_t raw[16];
                        tmem_ld16_async(trow + 16 * g, raw);
                        tmem_wait_ld16(raw);
#pragma unroll
                        for (int u = 0; u < 16; ++u) {
                            const int t = 16 * g + u;
                            if (t < nk && alive) {
                                const float djk =
                                    __fsub_rn(__fadd_rn(s_nrm[tid], k_nrm[t]), 2.f * __uint_as_float(raw[u]));
                                ++cc;
                                if (k_id[t] == id || occl(a.kind, a.t3, a.thr, k_pd[t], djk, pd)) alive = false;
                            }
                        }
                    }
                    fence_before();
                    __syncthreads(); // TMEM read by every warp before the next product
                    fence_after();
                }
                // 3. chunk x chunk: mask of earlier candidates that would occlude this one
                if (tid == 0) {
                    fence_after();
                    const uint32_t idesc = idesc_bf16(PT, PT);
                    for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                            mma_bf16(tmem, desc_sw128(tC + kb * PT * KBB + kk * 32),
                                     desc_sw128(tC + kb * PT * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
                    mma_commit(&bar_mma);
                }
                ok = mbar_wait(&bar_mma, ph_mma) && ok;
                ph_mma ^= 1u;
                fence_after();
                uint32_t mk[4] = {0u, 0u, 0u, 0u};
                {
                    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
                    const int gmax = (32 * warp + 31) >> 4; // groups holding columns < this warp's rows
#pragma unroll
                    for (int g = 0; g < PT / 16; ++g) {
                        if (g > gmax) break;
                        uint32_t raw[16];
                        tmem_ld16_async(trow + 16 * g, raw);
                        tmem_wait_ld16(raw);
#pragma unroll
                        for (int u = 0; u < 16; ++u) {
                            const int t = 16 * g + u;
                            if (t < tid && alive) {
                                const float djk =
                                    __fsub_rn(__fadd_rn(s_nrm[tid], s_nrm[t]), 2.f * __uint_as_float(raw[u]));
                                if (s_id[t] == id || occl(a.kind, a.t3, a.thr, s_pd[t], djk, pd))
                                    mk[t >> 5] |= 1u << (t & 31);
                            }
                        }
                    }
                }
#pragma unroll
                for (int x = 0; x < 4; ++x) s_mask[tid][x] = mk[x];
                const unsigned al = __ballot_sync(KCNA_FULL, alive);
                if (lane == 0) s_alive[warp] = al;
                fence_before();
                __syncthreads();
                fence_after();
                // 4. the scan, in candidate order, by warp 0: 32 candidates (one word
                // of the masks) at a time; lane p first tests the kept words of
                // earlier blocks, then the block is resolved in order with the
                // block's own mask word broadcast lane by lane
                if (warp == 0) {
                    uint32_t kw0 = 0u, kw1 = 0u, kw2 = 0u, kw3 = 0u; // kept chunk candidates
                    int nkl = nk, newk = 0;
                    for (int b = 0; b * 32 < m && nkl < a.range; ++b) {
                        const int p = 32 * b + lane;
                        const bool is_first = c0 + p == first;
                        const bool al_p = p < m && (is_first || ((s_alive[b] >> lane) & 1u));
                        const uint4 mk4 = *reinterpret_cast<const uint4 *>(s_mask[min(p, PT - 1)]);
                        const bool pre = ((mk4.x & kw0) | (mk4.y & kw1) | (mk4.z & kw2) | (mk4.w & kw3)) == 0u;
                        const uint32_t own = b == 0 ? mk4.x : b == 1 ? mk4.y : b == 2 ? mk4.z : mk4.w;
                        const unsigned cand = __ballot_sync(KCNA_FULL, al_p && pre);
                        uint32_t kb = 0u;
                        int cnt = nkl;
                        for (int i = 0; i < 32; ++i) {
                            const uint32_t wi = __shfl_sync(KCNA_FULL, own, i);
                            if (((cand >> i) & 1u) && !(wi & kb) && cnt < a.range) {
                                kb |= 1u << i;
                                ++cnt;
                            }
                        }
                        if ((kb >> lane) & 1u) {
                            const int r = __popc(kb & kcna_lanemask_lt());
                            k_id[nkl + r] = s_id[p];
                            k_pd[nkl + r] = s_pd[p];
                            k_nrm[nkl + r] = s_nrm[p];
                            s_kfrom[newk + r] = p;
                        }
                        if (b == 0) kw0 = kb;
                        if (b == 1) kw1 = kb;
                        if (b == 2) kw2 = kb;
                        if (b == 3) kw3 = kb;
                        nkl += __popc(kb);
                        newk += __popc(kb);
                    }
                    if (lane == 0) {
                        s_nk = nkl;
                        s_newk = newk;
                    }
                }
                __syncthreads();
                // 5. newly kept rows into the kept tile (rows nk.., swizzled like the chunk)
                const int newk = s_newk;
                for (int e = tid; e < newk * 2 * 8; e += PT) {
                    const int r = e >> 4, c16 = e & 15, kb = c16 >> 3, ch = c16 & 7;
                    const int src = s_kfrom[r], dst = nk + r;
                    const uint4 v = *reinterpret_cast<const uint4 *>(tiles + kb * PT * KBB + sw128_off((uint32_t)src, (uint32_t)ch));
                    *reinterpret_cast<uint4 *>(tiles + CHUNK + kb * KMAX * KBB + sw128_off((uint32_t)dst, (uint32_t)ch)) = v;
                }
                nk = s_nk;
                fence_proxy_async();
                __syncthreads();
                ok = __syncthreads_and(ok) != 0;
            }
        }
        // graph row of q
        for (int j = tid; j < (int)a.W; j += PT) {
            a.g_ids[(uint64_t)q * a.W + j] = j < nk ? k_id[j] : KCNA_NONE;
            a.g_dist[(uint64_t)q * a.W + j] = j < nk ? k_pd[j] : 0.f;
        }
        if (tid == 0) a.g_deg[q] = (uint32_t)nk;
        __syncthreads();
    }
    if (!ok && tid == 0) (void)mbar_wait(&bar_mma, ph_mma, 1u << 16); // a product still in flight
    cc = kcna_warp_sum(cc);
    if (lane == 0 && cc) atomicAdd(a.comps, cc);
    fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, TCOLS);
    if (!ok && tid == 0) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

} // namespace

bool kcna_prune_tc_ok(const kcna_ctx *c, int range) {
    return c->gram_exact && c->Xh && c->norms && !(c->ld & 7u) && c->ld <= 128 && range <= KMAX;
}

kcna_status kcna_prune_tc_launch(kcna_ctx *c, int kind, float t3, float thr, int range, int maxc,
                                 unsigned long long *comps) {
    if (!kcna_prune_tc_ok(c, range)) return kcna_fail(c, KCNA_E_STATE, "Gram-tile prune needs Gram-exact rows");
    PruneTcArgs a;
    a.N = c->n;
    a.cap = c->cap;
    a.W = c->W;
    a.pool = c->pool;
    a.pool_cnt = c->pool_cnt;
    a.norms = c->norms;
    a.kind = kind;
    a.t3 = t3;
    a.thr = thr;
    a.range = range;
    a.maxc = maxc;
    a.g_ids = c->g_ids;
    a.g_dist = c->g_dist;
    a.g_deg = c->g_deg;
    a.comps = comps;
    a.err = c->d_err;
    const size_t sm = 1024 + CHUNK + KEPT;
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(prune_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                             "prune_tc smem attr"));
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(prune_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                     (int)cudaSharedmemCarveoutMaxShared),
                             "prune_tc carveout"));
    int per_sm = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prune_tc_kernel, PT, sm),
                             "prune_tc occupancy"));
    per_sm = std::min(std::max(per_sm, 1), (int)(512 / TCOLS));
    const uint32_t grid = (uint32_t)std::min<uint64_t>(c->n, (uint64_t)std::max(c->num_sms, 1) * per_sm);
    alignas(64) CUtensorMap tmap;
    KCNA_TRY(kcna_rows_tmap(c, &tmap));
    prune_tc_kernel<<<grid, PT, sm, c->stream>>>(a, tmap, (int)c->ld);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "prune_tc_kernel");
}
