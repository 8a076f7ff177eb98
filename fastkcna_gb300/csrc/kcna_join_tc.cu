// kcna_join_tc.cu - NN-descent local join on tcgen05 Gram tiles.
//
// Same work as join_kernel (kcna_nnd.cu; reference join src/kgraph.cpp:1097-1117
// with Nhood::join :970-987): for node n, every pair of its new list A
// (i < j) and of A x old list B, each pair emitted to both endpoints'
// candidate buffers when within that endpoint's radius.  Here the distances
// come from Gram tiles: d(i, j) = (|x_i|^2 + |x_j|^2) - 2 <x_i, x_j>, with the
// dot products from tcgen05.mma on BF16 rows and FP32 accumulation in TMEM.
// The kernel runs only in Gram-exact mode (integer rows, squared norms below
// 2^23): every product and partial sum is then an integer below 2^24, so the
// tile distance is the canonical FMA-chain distance bit for bit and the join
// emits exactly the candidates of the FP32 kernel.
//
// Block layout: persistent, one block per SM, warp-specialised; the roles
// hand work to each other through mbarriers only, so no role waits for a
// block-wide barrier:
//   warp 0      producer: the bulk-copy engine brings node n+2's four lists
//               into a raw ring while node n is handled; assembles node n's
//               set (new list A, na <= 128, then the old list B; ncol entries)
//               in a node slot, gathers A's BF16 rows into the slot with TMA
//               (tile::gather4, 128-byte swizzle), then the set in tiles of 128
//               rows into a ring of row stages (freed as soon as the tile's
//               products are done) and the radius/norm of each row into a
//               deeper ring the epilogue frees; every gather lands as an
//               mbarrier arrival.
//   warp 1      MMA issuer (one thread): per tile, 4 (K=16) x 2 (64-element K
//               blocks) tcgen05.mma with M = 128 set rows and N = NA = na
//               rounded up to 16 new-list columns into one of four 128-column
//               TMEM accumulators; commits release the row stage and mark the
//               accumulator full.
//   warps 2-9   epilogue: warp w reads TMEM lanes 32*(w%4).. (set members) and
//               column groups of 16 of parity (w-2)/4; distance
//               |x|^2 + |y|^2 - 2<x,y>, pair rule of the reference join
//               (A x A with i < j, A x B); a set member's candidates are
//               counted per thread, a new member's by warp ballots; an
//               atomicAdd per target and tile reserves a contiguous run in the
//               target's candidate buffer (a row's run per column half, a
//               column's run per lane quarter: no barrier between epilogue
//               warps), the distances are read again from TMEM for the writes;
//               the last warp to finish a node writes its found flag.
// Every wait is bounded; a wait that gives up stops the block, sets the error
// word and lets in-flight products finish before TMEM is released.
#include <algorithm>

#include <cuda.h>

#include "kcna_internal.h"
#include "kcna_join.cuh"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int EPI_WARPS = 16;                 // epilogue warps: 4 per TMEM lane quarter
constexpr int WS_WARPS = 2 + EPI_WARPS;       // producer, MMA, epilogue
constexpr int WS_THREADS = WS_WARPS * 32;
constexpr int TROWS = 128;                    // set rows per tile (MMA M), max new-list columns
constexpr uint32_t KBB = 128;                 // bytes of a row inside one 64-element K block
constexpr uint32_t TILE = TROWS * KBB * 2;    // 128 rows, two K blocks (d <= 128): 32 KiB
constexpr int NS = 2;                         // node slots
constexpr int TS = 3;                         // tile row stages (released by the MMA)
constexpr int MS = 6;                         // tile metadata entries (released by the epilogue)
constexpr int NACC = 4;                       // TMEM accumulators of 128 columns
constexpr int NR = 4;                         // raw list entries (prefetched two nodes ahead)

// Layout of one raw list entry: the four lists of a node copied whole.
struct RawLayout {
    uint32_t o_rnew, o_old, o_rold, words; // offsets (in u32) after the forward-new list
};
__host__ __device__ inline RawLayout raw_layout(uint32_t fwd_new_cap, uint32_t rc, uint32_t fwd_old_cap) {
    RawLayout r;
    r.o_rnew = fwd_new_cap;
    r.o_old = r.o_rnew + rc;
    r.o_rold = r.o_old + fwd_old_cap;
    r.words = r.o_rold + rc;
    return r;
}

struct SlotMeta {
    uint32_t node, na, NA, ncol;
};

// Shared-memory carve-up (after the 1024-aligned tiles: NS slots + TS stages)
struct WsShared {
    uint64_t node_full[NS], node_empty[NS], tile_full[TS], tile_empty[TS], meta_full[MS], meta_empty[MS];
    uint64_t acc_full[NACC], acc_empty[NACC], ids_full[NR];
    SlotMeta meta[NS];
    uint32_t tmem;
    volatile int abort_flag;
    unsigned emit[NS], done[NS];
    float a_rad[NS][TROWS], a_nrm[NS][TROWS];
    float t_rad[MS][TROWS], t_nrm[MS][TROWS];
    // screening bound terms (BF16 screen mode): sqrt(radius (1 + 2^-15)) and
    // the norm of the rounded row
    float a_rr[NS][TROWS], a_aa[NS][TROWS], t_rr[MS][TROWS], t_aa[MS][TROWS];
};

// rows [first, first+count) of ids -> rows 0..count-1 of a 128-row region by
// TMA gather4 (four rows of one K block per instruction; the last group
// repeats its last row), lane-strided.  Returns the transaction bytes.
__device__ __forceinline__ uint32_t tma_rows(uint32_t region, const uint32_t *ids, int first, int count,
                                             const void *tmap, int nkb, uint64_t *bar, int lane) {
    const int ng = (count + 3) >> 2;
    for (int e = lane; e < ng * nkb; e += 32) {
        const int g = nkb == 2 ? e >> 1 : e, kb = nkb == 2 ? e & 1 : 0;
        const int r = 4 * g, last = first + count - 1;
        tma_gather4(region + (uint32_t)kb * TROWS * KBB + (uint32_t)r * KBB, tmap, 64 * kb, (int)ids[first + r],
                    (int)ids[min(first + r + 1, last)], (int)ids[min(first + r + 2, last)],
                    (int)ids[min(first + r + 3, last)], bar);
    }
    return (uint32_t)(ng * 4 * nkb) * KBB;
}

// D[128 x N] = rows(a) . rows(b)^T over nkb K blocks of 64 elements.
__device__ __forceinline__ void issue_tile(uint32_t tmem_d, uint32_t a_base, uint32_t b_base, uint32_t idesc,
                                           int nkb) {
    for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma_bf16(tmem_d, desc_sw128(a_base + kb * TROWS * KBB + kk * 32),
                     desc_sw128(b_base + kb * TROWS * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
}

// Screening bound of a rounded-row Gram distance (BF16 screen mode): with
// x~ the rows rounded to BF16 (relative error <= 2^-8 per element), a pair
// whose FP32 distance is <= radius has Gram distance
//   ds <= (sqrt(radius (1 + 2^-15)) + 2^-7 (|x~_i| + |x~_j|))^2 + 2^-14 (|x~_i|^2 + |x~_j|^2)
// (rounding of the rows, of the FP32 chain and of the FP32 accumulation, each
// bound doubled).  Pairs below the bound are emitted and recomputed in FP32.
constexpr float SCREEN_CE = 0.0078125f;     // 2^-7
constexpr float SCREEN_CG = 6.103515625e-05f; // 2^-14
__device__ __forceinline__ float screen_bound(float rr, float aa_sum, float nn_sum) {
    const float t = __fmaf_rn(SCREEN_CE, aa_sum, rr);
    return __fmaf_rn(t, t, SCREEN_CG * nn_sum);
}

template <bool SCREEN>
__global__ void __launch_bounds__(WS_THREADS, 1) join_tc_kernel(JoinArgs a, const __grid_constant__ CUtensorMap tmap,
                                                                int ldh, const float *__restrict__ norms,
                                                                const float *__restrict__ rr,
                                                                const float *__restrict__ aa, uint32_t colcap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u; // swizzled tiles need 1024-byte alignment
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    WsShared &S = *reinterpret_cast<WsShared *>(tiles + (NS + TS) * TILE);
    uint32_t *set_ids = reinterpret_cast<uint32_t *>(&S + 1); // NS x colcap
    // raw list ring: NR entries, 16-byte aligned
    const uint32_t rc = (min(a.R, a.RB) + 3) & ~3u;
    const RawLayout RL = raw_layout(a.fwd_new_cap, rc, a.fwd_old_cap);
    uint32_t *raw_ring = reinterpret_cast<uint32_t *>(
        (reinterpret_cast<uintptr_t>(set_ids + (size_t)NS * colcap) + 15) & ~(uintptr_t)15);
    const uint32_t slotA = tiles_s, stage0 = tiles_s + NS * TILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = (ldh + 63) >> 6;
    const void *tm = &tmap;

    // K padding beyond ldh is never written by the gathers and must read as zero
    for (int i = tid; i < (int)((NS + TS) * TILE / 16); i += WS_THREADS)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 1) tmem_alloc(&S.tmem, NACC * TROWS);
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(&S.node_full[i], 33);  // 32 producer lanes' copies + the producer's expect_tx (metadata, A rows)
            mbar_init(&S.node_empty[i], EPI_WARPS);
            S.emit[i] = 0;
            S.done[i] = 0;
        }
        for (int i = 0; i < TS; ++i) {
            mbar_init(&S.tile_full[i], 1);   // producer's expect_tx; the TMA gathers complete it
            mbar_init(&S.tile_empty[i], 1);  // MMA commit
        }
        for (int i = 0; i < MS; ++i) {
            mbar_init(&S.meta_full[i], 32);  // producer lanes' copies
            mbar_init(&S.meta_empty[i], EPI_WARPS);
        }
        for (int i = 0; i < NR; ++i) mbar_init(&S.ids_full[i], 1); // producer's expect_tx + bulk copies
        for (int i = 0; i < NACC; ++i) {
            mbar_init(&S.acc_full[i], 1);    // MMA commit
            mbar_init(&S.acc_empty[i], EPI_WARPS);
        }
        S.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        unsigned long long pairs = 0, rows_g = 0;
        uint32_t tcount = 0;
        // the four lists of node number kk (grid-stride) copied whole by the
        // bulk-copy engine into raw entry kk % NR; lane 0 issues
        auto prefetch = [&](int kk) {
            const uint32_t nd = blockIdx.x + (uint32_t)kk * gridDim.x;
            if (nd >= a.N || lane != 0) return;
            uint32_t *r = raw_ring + (size_t)(kk % NR) * RL.words;
            uint64_t *bar = &S.ids_full[kk % NR];
            const uint32_t bytes = RL.words * 4 - (a.iter > 0 ? 0u : 2u * rc * 4);
            mbar_arrive_expect_tx(bar, bytes);
            bulk_copy_g2s(smem_u32(r), a.fwd_new + (uint64_t)nd * a.fwd_new_cap, a.fwd_new_cap * 4, bar);
            bulk_copy_g2s(smem_u32(r + RL.o_old), a.fwd_old + (uint64_t)nd * a.fwd_old_cap, a.fwd_old_cap * 4, bar);
            if (a.iter > 0) {
                bulk_copy_g2s(smem_u32(r + RL.o_rnew), a.rnew + (uint64_t)nd * a.RB, rc * 4, bar);
                bulk_copy_g2s(smem_u32(r + RL.o_rold), a.rold + (uint64_t)nd * a.RB, rc * 4, bar);
            }
        };
        // list lengths, loaded two nodes ahead into registers
        uint32_t c_fn[3] = {0, 0, 0}, c_rn[3] = {0, 0, 0}, c_fo[3] = {0, 0, 0}, c_ro[3] = {0, 0, 0};
        auto load_counts = [&](int kk, int slot) { // raw values; clamped where used
            const uint32_t nd = blockIdx.x + (uint32_t)kk * gridDim.x;
            if (nd >= a.N) return;
            c_fn[slot] = a.fwd_new_cnt[nd];
            c_fo[slot] = a.fwd_old_cnt[nd];
            if (a.iter > 0) {
                c_rn[slot] = a.rnew_cnt[nd];
                c_ro[slot] = a.rold_cnt[nd];
            }
        };
        prefetch(0);
        prefetch(1);
        load_counts(0, 0);
        load_counts(1, 1);
        int k = 0;
        for (uint32_t node = blockIdx.x; node < a.N; node += gridDim.x, ++k) {
            const int sl = k & 1;
            const uint32_t fn = min(c_fn[0], a.fwd_new_cap), rn = a.iter > 0 ? min(c_rn[0], a.R) : 0u;
            const uint32_t fo = min(c_fo[0], a.fwd_old_cap), ro = a.iter > 0 ? min(c_ro[0], a.R) : 0u;
            c_fn[0] = c_fn[1], c_rn[0] = c_rn[1], c_fo[0] = c_fo[1], c_ro[0] = c_ro[1];
            c_fn[1] = c_fn[2], c_rn[1] = c_rn[2], c_fo[1] = c_fo[2], c_ro[1] = c_ro[2];
            load_counts(k + 2, 1);
            if (!mbar_wait(&S.ids_full[k % NR], (k / NR) & 1)) { ok = false; break; }
            if (k >= NS && !mbar_wait(&S.node_empty[sl], ((k >> 1) - 1) & 1)) { ok = false; break; }
            if (S.abort_flag) break;
            // compact the node's set from its raw entry: A (new list, <= 128), then B
            const uint32_t *raw = raw_ring + (size_t)(k % NR) * RL.words;
            uint32_t *ids = set_ids + (size_t)sl * colcap;
            const uint32_t na = min(fn + rn, (uint32_t)TROWS);
            const uint32_t ncol = na + fo + ro;
            for (uint32_t i = lane; i < fn && i < na; i += 32) ids[i] = raw[i];
            for (uint32_t i = lane; i < rn && fn + i < na; i += 32) ids[fn + i] = raw[RL.o_rnew + i];
            for (uint32_t i = lane; i < fo; i += 32) ids[na + i] = raw[RL.o_old + i];
            for (uint32_t i = lane; i < ro; i += 32) ids[na + fo + i] = raw[RL.o_rold + i];
            __syncwarp();
            prefetch(k + 2); // raw entry (k+2) % NR was compacted two nodes ago
            if (lane == 0) {
                S.meta[sl].node = node;
                S.meta[sl].na = na;
                S.meta[sl].NA = (na + 15) & ~15u;
                S.meta[sl].ncol = ncol;
                if (na) {
                    pairs += (unsigned long long)na * (na - 1) / 2 + (unsigned long long)na * (ncol - na);
                    rows_g += ncol;
                }
            }
            for (uint32_t i = lane; i < na; i += 32) {
                cp_async4(smem_u32(&S.a_rad[sl][i]), a.radius + ids[i]);
                cp_async4(smem_u32(&S.a_nrm[sl][i]), norms + ids[i]);
                if (SCREEN) {
                    cp_async4(smem_u32(&S.a_rr[sl][i]), rr + ids[i]);
                    cp_async4(smem_u32(&S.a_aa[sl][i]), aa + ids[i]);
                }
            }
            // padding columns na..NA-1: a NaN norm makes every distance NaN, so no pair passes
            for (uint32_t i = na + lane; i < ((na + 15) & ~15u); i += 32) {
                S.a_nrm[sl][i] = __uint_as_float(0x7FC00000u);
                S.a_rad[sl][i] = 0.f;
            }
            mbar_arrive_cp_async(&S.node_full[sl]);
            __syncwarp();
            if (lane == 0) mbar_arrive_expect_tx(&S.node_full[sl], (uint32_t)((na + 3) / 4 * 4 * nkb) * KBB);
            __syncwarp();
            if (na) tma_rows(slotA + sl * TILE, ids, 0, (int)na, tm, nkb, &S.node_full[sl], lane);
            const int ntile = na ? (int)((ncol + TROWS - 1) / TROWS) : 0;
            for (int t = 0; t < ntile; ++t, ++tcount) {
                const int st = (int)(tcount % TS), mt = (int)(tcount % MS);
                if (tcount >= (uint32_t)MS && !mbar_wait(&S.meta_empty[mt], ((tcount / MS) - 1) & 1)) {
                    ok = false;
                    break;
                }
                const int first = t * TROWS, cnt = min((int)ncol - first, TROWS);
                for (int i = lane; i < cnt; i += 32) {
                    cp_async4(smem_u32(&S.t_rad[mt][i]), a.radius + ids[first + i]);
                    cp_async4(smem_u32(&S.t_nrm[mt][i]), norms + ids[first + i]);
                    if (SCREEN) {
                        cp_async4(smem_u32(&S.t_rr[mt][i]), rr + ids[first + i]);
                        cp_async4(smem_u32(&S.t_aa[mt][i]), aa + ids[first + i]);
                    }
                }
                mbar_arrive_cp_async(&S.meta_full[mt]);
                if (tcount >= (uint32_t)TS && !mbar_wait(&S.tile_empty[st], ((tcount / TS) - 1) & 1)) {
                    ok = false;
                    break;
                }
                if (lane == 0) mbar_arrive_expect_tx(&S.tile_full[st], (uint32_t)((cnt + 3) / 4 * 4 * nkb) * KBB);
                __syncwarp();
                tma_rows(stage0 + st * TILE, ids, first, cnt, tm, nkb, &S.tile_full[st], lane);
            }
            if (!ok) break;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        // bulk copies still in flight (prefetched lists of nodes not processed) land before exit
        for (int kk = k; kk <= k + 2; ++kk) {
            const uint32_t nd = blockIdx.x + (uint32_t)kk * gridDim.x;
            if (nd < a.N) (void)mbar_wait(&S.ids_full[kk % NR], (kk / NR) & 1, 1u << 16);
        }
        if (!ok) S.abort_flag = 1;
        if (lane == 0) {
            atomicAdd(a.counters + 0, pairs);
            atomicAdd(a.counters + 5, rows_g);
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            uint32_t tcount = 0, acount = 0;
            int k = 0;
            for (uint32_t node = blockIdx.x; node < a.N; node += gridDim.x, ++k) {
                const int sl = k & 1;
                if (!mbar_wait(&S.node_full[sl], (k >> 1) & 1) || S.abort_flag) { ok = false; break; }
                const uint32_t na = S.meta[sl].na, NA = S.meta[sl].NA, ncol = S.meta[sl].ncol;
                const int ntile = na ? (int)((ncol + TROWS - 1) / TROWS) : 0;
                const uint32_t idesc = idesc_bf16(TROWS, (int)NA);
                for (int t = 0; t < ntile; ++t, ++tcount, ++acount) {
                    const int st = (int)(tcount % TS), b = (int)(acount % NACC);
                    if (!mbar_wait(&S.tile_full[st], (tcount / TS) & 1)) { ok = false; break; }
                    if (acount >= (uint32_t)NACC && !mbar_wait(&S.acc_empty[b], ((acount / NACC) - 1) & 1)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    issue_tile(tmem + (uint32_t)(b * TROWS), stage0 + st * TILE, slotA + sl * TILE, idesc, nkb);
                    mma_commit(&S.acc_full[b]);
                    mma_commit(&S.tile_empty[st]);
                }
                if (!ok) break;
            }
            if (!ok) {
                S.abort_flag = 1;
                // products still in flight finish before TMEM is released
                for (uint32_t b = 0; b < (uint32_t)NACC; ++b)
                    if (acount > b) {
                        const uint32_t last = b + (acount - 1 - b) / NACC * NACC; // last tile issued to b
                        (void)mbar_wait(&S.acc_full[b], (last / NACC) & 1u, 1u << 16);
                    }
            }
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3, h = (warp - 2) >> 2; // TMEM lane quarter, column-group phase (0..3)
        const int rw = 32 * q + lane;                // this thread's row of a tile
        unsigned long long emitted = 0;
        uint32_t tcount = 0;
        int k = 0;
        for (uint32_t node = blockIdx.x; node < a.N; node += gridDim.x, ++k) {
            const int sl = k & 1;
            bool mine = mbar_wait(&S.node_full[sl], (k >> 1) & 1) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            const int na = (int)S.meta[sl].na, NA = (int)S.meta[sl].NA, ncol = (int)S.meta[sl].ncol;
            const int G = NA >> 4;
            const int ntile = na ? (ncol + TROWS - 1) / TROWS : 0;
            const uint32_t *ids = set_ids + (size_t)sl * colcap;
            const float *arad = S.a_rad[sl], *anrm = S.a_nrm[sl]; // anrm is NaN on columns na..NA-1
            for (int t = 0; t < ntile; ++t, ++tcount) {
                const int mt = (int)(tcount % MS), b = (int)(tcount % NACC);
                mine = mbar_wait(&S.acc_full[b], (tcount / NACC) & 1) && mbar_wait(&S.meta_full[mt], (tcount / MS) & 1);
                fence_after();
                const int j = t * TROWS + rw; // set member
                const bool warp_live = t * TROWS + 32 * q < ncol && h < G;
                const bool rowv = j < ncol && mine;
                const uint32_t id_j = rowv ? ids[j] : 0u;
                const float rad_j = rowv ? S.t_rad[mt][rw] : 0.f;
                const float n_j = rowv ? S.t_nrm[mt][rw] : __uint_as_float(0x7FC00000u); // NaN: no pair passes
                const float rr_j = SCREEN && rowv ? S.t_rr[mt][rw] : 0.f, aa_j = SCREEN && rowv ? S.t_aa[mt][rw] : 0.f;
                const float *arr = S.a_rr[sl], *aaa = S.a_aa[sl];
                // rows of the new list meet only earlier new-list columns (each pair once)
                const bool tri = t == 0 && 32 * q < na;
                const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * TROWS);
                uint32_t rmask = 0, cm = 0; // cm: ballot of local column `lane`
                if (warp_live) {
#pragma unroll 1
                    for (int kk = 0; kk < 2; ++kk) {
                        const int g = h + 4 * kk;
                        if (g >= G) break;
                        uint32_t raw[16];
                        tmem_ld16_async(trow + 16 * g, raw);
                        tmem_wait_ld16(raw);
#pragma unroll
                        for (int u = 0; u < 16; ++u) {
                            const int i = 16 * g + u; // new-list column
                            const float nn = __fadd_rn(n_j, anrm[i]);
                            const float dd = __fsub_rn(nn, 2.f * __uint_as_float(raw[u]));
                            bool rp, cp;
                            if (SCREEN) {
                                const float as = __fadd_rn(aa_j, aaa[i]);
                                rp = dd <= screen_bound(rr_j, as, nn);
                                cp = dd <= screen_bound(arr[i], as, nn);
                            } else {
                                rp = dd <= rad_j;
                                cp = dd <= arad[i];
                            }
                            if (tri && i >= j) rp = cp = false;
                            if ((rp || cp) && ids[i] == id_j) rp = cp = false; // an id in both lists
                            rmask |= (uint32_t)rp << (16 * kk + u);
                            const unsigned m = __ballot_sync(KCNA_FULL, cp);
                            if (lane == 16 * kk + u) cm = m;
                        }
                    }
                }
                // reservations without barriers between warps: each thread
                // reserves its row's run for this warp's columns, lane c the
                // run of local column c for this lane quarter
                const int nr = __popc(rmask), nc = __popc(cm);
                uint32_t p = nr ? atomicAdd(a.cand_cnt + id_j, (uint32_t)nr) : 0u;
                const uint32_t cb =
                    nc ? atomicAdd(a.cand_cnt + ids[16 * (h + 4 * (lane >> 4)) + (lane & 15)], (uint32_t)nc) : 0u;
                const unsigned wtot = kcna_warp_sum((unsigned)(nr + nc));
                if (lane == 0 && wtot) atomicAdd(&S.emit[sl], wtot);
                if (wtot) { // writes; the distances are read again from TMEM
                    const uint32_t flags = (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW);
                    uint64_t *dst = a.cand + (uint64_t)id_j * a.CB;
#pragma unroll 1
                    for (int kk = 0; kk < 2; ++kk) {
                        const int g = h + 4 * kk;
                        if (g >= G) break;
                        const uint32_t gm = (rmask >> (16 * kk)) & 0xFFFFu;
                        const uint32_t cmk = (lane >> 4) == kk ? cm : 0u;
                        if (!__any_sync(KCNA_FULL, gm != 0u || cmk != 0u)) continue;
                        uint32_t raw[16];
                        tmem_ld16_async(trow + 16 * g, raw);
                        tmem_wait_ld16(raw);
#pragma unroll
                        for (int u = 0; u < 16; ++u) {
                            const int i = 16 * g + u;
                            const int c = 16 * kk + u;
                            const unsigned m = __shfl_sync(KCNA_FULL, cm, c);
                            const uint32_t cbc = __shfl_sync(KCNA_FULL, cb, c);
                            if (((gm >> u) & 1u) || ((m >> lane) & 1u)) {
                                // emitted with the Gram distance (exact in Gram-exact mode;
                                // recomputed in FP32 by the rescore in screen mode)
                                const float dd = fmaxf(
                                    __fsub_rn(__fadd_rn(n_j, anrm[i]), 2.f * __uint_as_float(raw[u])), 0.f);
                                if ((gm >> u) & 1u) {
                                    if (p < a.CB) dst[p] = kcna_key(dd, ids[i], flags);
                                    ++p;
                                }
                                if ((m >> lane) & 1u) {
                                    const uint32_t pc = cbc + __popc(m & kcna_lanemask_lt());
                                    if (pc < a.CB) a.cand[(uint64_t)ids[i] * a.CB + pc] = kcna_key(dd, id_j, flags);
                                }
                            }
                        }
                    }
                }
                if (!mine) ok = false;
                // accumulator and metadata entry released by each epilogue warp
                fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&S.acc_empty[b]);
                    mbar_arrive(&S.meta_empty[mt]);
                }
                if (!__all_sync(KCNA_FULL, ok)) {
                    ok = false;
                    break;
                }
            }
            if (!ok) break;
            // found: this node's join emitted a candidate; the last epilogue
            // warp to finish the node writes it
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                if (atomicAdd(&S.done[sl], 1u) == (unsigned)(EPI_WARPS - 1)) {
                    __threadfence_block();
                    const unsigned e = atomicExch(&S.emit[sl], 0u);
                    if (na > 0) a.found[S.meta[sl].node] = e ? 1 : 0;
                    emitted += e;
                    S.done[sl] = 0;
                }
                mbar_arrive(&S.node_empty[sl]);
            }
        }
        if (!ok) S.abort_flag = 1;
        if (lane == 0 && emitted) atomicAdd(a.counters + 6, emitted);
    }
    fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, NACC * TROWS);
    if (!ok) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

} // namespace

static size_t join_tc_smem(const JoinArgs &a) {
    const uint32_t colcap = std::max<uint32_t>(a.capA, TROWS + a.capB);
    const uint32_t rc = (std::min(a.R, a.RB) + 3) & ~3u;
    const RawLayout RL = raw_layout(a.fwd_new_cap, rc, a.fwd_old_cap);
    return 1024 + (size_t)(NS + TS) * TILE + sizeof(WsShared) + (size_t)NS * colcap * 4 + 16 + (size_t)NR * RL.words * 4;
}

bool kcna_join_tc_fits(const JoinArgs &a) {
    return join_tc_smem(a) <= 227 * 1024 && !((a.fwd_new_cap | a.fwd_old_cap | a.RB) & 3u);
}

// sqrt(radius (1 + 2^-15)) and sqrt(norm) for the screening bound
__global__ void screen_terms_kernel(const float *__restrict__ radius, const float *__restrict__ norms, uint32_t n,
                                    float *__restrict__ rr, float *__restrict__ aa) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rr[i] = __fsqrt_ru(__fmul_ru(radius[i], 1.000030517578125f));
    aa[i] = __fsqrt_ru(norms[i]);
}

kcna_status kcna_join_tc_launch(kcna_ctx *c, const JoinArgs &a) {
    if (!(c->gram_exact || c->bf16_screen) || !c->Xh || !c->norms || (c->ld & 7u) || c->ld > 128)
        return kcna_fail(c, KCNA_E_STATE, "Gram-tile join needs BF16 rows with d <= 128");
    const uint32_t colcap = std::max<uint32_t>(a.capA, TROWS + a.capB);
    if (!kcna_join_tc_fits(a)) return kcna_fail(c, KCNA_E_STATE, "Gram-tile join: lists too long for shared memory");
    const size_t sm = join_tc_smem(a);
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "join_tc smem attr"));
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "join_tc smem attr"));
    const uint32_t grid = (uint32_t)std::min<uint64_t>(a.N, (uint64_t)std::max(c->num_sms, 1));
    if (grid == 0) return KCNA_OK;
    alignas(64) CUtensorMap tmap;
    KCNA_TRY(kcna_rows_tmap(c, &tmap));
    if (c->bf16_screen) {
        float *rr = nullptr, *aa = nullptr;
        KCNA_TRY(kcna_scratch(c, (size_t)c->n * 8, reinterpret_cast<void **>(&rr)));
        aa = rr + c->n;
        screen_terms_kernel<<<kcna_div_up(c->n, 256), 256, 0, c->stream>>>(a.radius, c->norms, c->n, rr, aa);
        KCNA_LAUNCHED(c);
        join_tc_kernel<true><<<grid, WS_THREADS, sm, c->stream>>>(a, tmap, (int)c->ld, c->norms, rr, aa, colcap);
    } else {
        join_tc_kernel<false><<<grid, WS_THREADS, sm, c->stream>>>(a, tmap, (int)c->ld, c->norms, nullptr, nullptr,
                                                                  colcap);
    }
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "join_tc_kernel");
}
