// kcna_prune_tc.cu - occlusion prune on tcgen05 Gram tiles.
//
// Same result as prune_kernel (kcna_graph.cu; reference nsg_sync_prune
// src/kgraph.cpp:1809-1851, taumg_sync_prune :2833-2876, alphapg_sync_prune
// :3157-3203) for the RNG, tau-MNG and alpha-PG rules: the candidates of node
// q are pool[first .. lim) in order; the first is kept; a later candidate p
// is dropped when an already kept t occludes it (RNG: d(t,p) < d(q,p);
// tau-MNG: d(t,p) < d(q,p) - 3 tau; alpha-PG: d(t,p) < d(q,p) and the angle
// at t below the threshold angle), and the scan stops at range kept.  The kernel runs only in Gram-exact mode (integer rows, squared norms
// below 2^23), where the tile distances (|x|^2 + |y|^2) - 2 <x, y> (BF16
// rows, FP32 accumulation in TMEM) equal the canonical FMA-chain distances,
// so the kept lists are identical.
//
// Instead of testing candidates against the kept list one at a time, the
// kernel evaluates the occlusion rule for every ordered pair t < p of the
// node's candidates (up to 512: the lower triangle of at most 4 x 4 tiles of
// 128) and then resolves the sequential scan on bit masks: O[t] is the set of
// later candidates that t would occlude, and the scan keeps t, adds O[t] to
// the dead set and jumps to the next live candidate - one step per kept
// neighbour.
//
// Block layout: persistent, one block per SM, warp-specialised; the roles
// hand work to each other through mbarriers:
//   warp 0      metadata: node q's pool prefix by one bulk copy (requested a
//               node ahead), the initial dead set (ids beyond the layer
//               prefix, repeated ids), distances, and the candidates' norms by
//               4-byte cp.async (two nodes in flight);
//   warps 19-22 row loaders: the candidates' BF16 rows by 16-byte cp.async
//               into a ring of five 128-row chunk slots in the 128-byte
//               swizzled K-major layout (each warp a quarter of every chunk,
//               the copies of consecutive chunks overlapped);
//   warp 1      MMA issuer (one thread): tiles (J, I), J <= I, occluders of
//               chunk J (M = 128 TMEM lanes) against candidates of chunk I
//               (N = 128 columns), occluder-chunk major so that chunk J's slot
//               is released after its last tile; four 128-column accumulators;
//   warps 2-17  mask builders: warp w reads TMEM lane quarter w % 4 and
//               column group (w - 2) / 4 (32 columns) of a tile, releases the
//               accumulator, and turns 32 distances per thread into a 32-bit
//               word of O[t] (the sign of distance minus bound, collected by
//               funnel shifts in four independent chains);
//   warp 18     scan: per node, the kept list by the bit-mask scan; graph row
//               and degree written to global memory.
// Every wait is bounded; a wait that gives up stops the block, sets the error
// word and lets in-flight copies and products finish before TMEM is released.
#include <algorithm>

#include "kcna_internal.h"
#include "kcna_tc.cuh"

using namespace kcna_tc;

namespace {

constexpr int PC = 128;                           // candidates per chunk (MMA M and N)
constexpr int MAXCH = 4;                          // chunks per node
constexpr int MAXC = PC * MAXCH;                  // candidates per node
constexpr int MW = MAXC / 32;                     // mask words per row
constexpr uint32_t KBB = 128;                     // bytes of a row inside one 64-element K block
constexpr uint32_t CHUNK_BYTES = PC * KBB * 2;    // 128 rows, two K blocks (d <= 128): 32 KiB
constexpr int NSLOT = 5;                          // chunk slots (>= MAXCH)
constexpr int NACC = 4;                           // 128-column TMEM accumulators
constexpr int EPI = 16;                           // mask-building warps: 4 lane quarters x 4 column groups
constexpr int CW = PC / (EPI / 4);                // columns of a tile per mask-building warp
constexpr int WPT = CW / 32;                      // mask words per thread and tile
constexpr int SCAN_WARP = 2 + EPI;
constexpr int LOAD_WARP = SCAN_WARP + 1;          // first row-loader warp
constexpr int NLOAD = 4;                          // row-loader warps
constexpr int PG_THREADS = (LOAD_WARP + NLOAD) * 32;

// Occluder masks, word-major: word w (candidates 32w .. 32w+31) of row t is at
// mask_base(w) + t; word w exists for rows t < 128 (w / 4 + 1) only (t < p).
// mask_base(w) is w modulo 32, so both the mask builders (fixed w, 32
// consecutive t) and the scan (fixed t, 16 words) are free of bank conflicts.
__host__ __device__ constexpr int mask_base(int w) {
    return 128 * ((w / 4) * (w / 4 + 1) / 2 * 4 + (w % 4) * (w / 4 + 1)) + w;
}
constexpr int MASK_WORDS = mask_base(MW);

struct alignas(16) NodeMeta {
    uint64_t key[MAXC + 2]; // pool entries from an even index (16-byte bulk copy); candidate c at koff + c
    float pd[MAXC];         // distance to the node
    float nrm[MAXC];        // squared norm of the row
    uint32_t dead[MW];      // candidates that can never be kept
    uint32_t q, nc, nch, koff;
};

struct PgShared {
    uint64_t slot_full[NSLOT], slot_empty[NSLOT];
    uint64_t acc_full[NACC], acc_empty[NACC];
    uint64_t keys_full[2], ids_ready[2], meta_full[2], bound_ready[2], mask_full[2], node_empty[2];
    uint32_t tmem;
    volatile int abort_flag;
    NodeMeta meta[2];
    uint32_t mask[2][MASK_WORDS];
};

struct PgArgs {
    uint32_t N, cap, W, ld; // N: ids at or beyond are skipped (the layer prefix); cap: candidate row stride
    uint32_t n_items;       // nodes (or staged lists) to prune
    const uint32_t *nodes;  // staged lists: node of list k (null: item k is node k)
    uint32_t by_node;       // 1: item k is the pool of node nodes[k] (candidate row nodes[k])
    const uint64_t *pool;   // candidate keys, row = node (or list), cap apart
    const uint16_t *rows;   // BF16 rows, ld elements apart
    const uint32_t *pool_cnt; // candidates of each row
    const float *norms;
    float aux, thr; // aux: 3 tau (tau-MNG) or the angle screen's margin 4m (alpha-PG)
    int range, maxc;
    uint32_t *g_ids;
    float *g_dist;
    uint32_t *g_deg;
    unsigned long long *comps;
    int *err;
};

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
// wait_group covers committed groups only: commit whatever is outstanding first
__device__ __forceinline__ void cp_async_wait_0() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// A word whose sign bit says whether t occludes p, from the Gram entry g:
// |t|^2 - 2g + |p|^2 is exact in Gram-exact mode, and the sign of its
// difference to the bound is the result of the FP32 comparison.  For RNG the
// column value is pd - |p|^2 (an exact integer difference in Gram-exact mode:
// pool distances are canonical distances of integer rows), one add fewer.
// The alpha-PG angle test exactly as the FP32 prune and the reference evaluate
// it (src/kgraph.cpp:3181-3183): cos = ((td + djk) - pd) / 2 / sqrt(td * djk),
// IEEE operations in that order, compared with the FP32 threshold.
__device__ __noinline__ bool alpha_angle_exact(float td, float djk, float pd, float thr) {
    const float num = __fdiv_rn(__fsub_rn(__fadd_rn(td, djk), pd), 2.0f);
    const float cs = __fdiv_rn(num, __fsqrt_rn(__fmul_rn(td, djk)));
    return cs < thr;
}

// alpha-PG (RULE 2) without the angle arithmetic on almost every pair.  The
// candidates are sorted by distance to the node, so a = d(q,t) <= c = d(q,p),
// and the occlusion needs b = d(t,p) < c: qp is then the longest side of the
// triangle q, t, p and the angle at t its largest, at least 60 degrees.  With
// x = 1 - a/c, y = 1 - b/c and s = x + y = (2c - a - b) / c,
//   cos(t) = (1 - s) / (2 sqrt((1 - x)(1 - y))),
// and for s < 1 the root is at least sqrt(1 - s) ((1 - x)(1 - y) = 1 - s + xy),
// so cos(t) <= sqrt(1 - s) / 2 <= 1/2 - s/4; for s >= 1, cos(t) <= 0.  With
// the threshold thr = cos(angle) >= cos(60 degrees) and m = 1/2 - thr + 1e-5
// (the 1e-5 covers the few-ulp error of the FP32 formula: Gram-exact distances
// are integers, so a nonzero side is at least 1), s > 4m proves cos(t) < thr
// and the pair is occluded as under RNG.  Only near-equilateral pairs
// (2c - a - b within 4m c + 16 of zero, alpha_signs below) and pairs with
// b = 0 (duplicate rows: the formula's 0/0 is NaN, not occluded) take the
// exact test.

// A word whose sign bit says whether t occludes p, from the Gram entry g:
// |t|^2 - 2g + |p|^2 is exact in Gram-exact mode, and the sign of its
// difference to the bound is the result of the FP32 comparison.  For RNG the
// column value is pd - |p|^2 (an exact integer difference in Gram-exact mode:
// pool distances are canonical distances of integer rows), one add fewer.
template <int RULE>
__device__ __forceinline__ uint32_t occl_sign(float g, float nt, float np, float pd, float aux) {
    if (RULE == 0) return __float_as_uint(__fsub_rn(__fmaf_rn(-2.f, g, nt), pd)); // pd holds pd - |p|^2
    const float dd = __fadd_rn(__fmaf_rn(-2.f, g, nt), np);
    return __float_as_uint(__fsub_rn(dd, __fsub_rn(pd, aux))); // src/kgraph.cpp:2859
}

// alpha-PG (RULE 2): three sign words per 32 pairs, branch-free.  With a =
// td, c = pd and b = dd (integers in Gram-exact mode):
//   r: b < c                                   (the RNG part of the rule)
//   o: b < min(c, (2 - 4m) c - 16 - a)         (the screen: 2c - a - b > 4m c
//      with room for the FMA's rounding, at most 4; m <= c, so o implies r)
//   z: b > 1/2                                 (no zero side: the formula's 0/0)
// o & z: proven occluded; r & ~(o & z): the exact test.  A zero a needs no
// test: the formula then gives -inf, occluded whenever b < c.  k2 = 2 - 4m,
// ctd = -16 - a (per row).
__device__ __forceinline__ void alpha_signs(float g, float nt, float np, float pd, float k2, float ctd, uint32_t &r,
                                            uint32_t &o, uint32_t &z) {
    const float dd = __fadd_rn(__fmaf_rn(-2.f, g, nt), np);
    const float m = fminf(pd, __fmaf_rn(k2, pd, ctd));
    r = __float_as_uint(__fsub_rn(dd, pd));
    o = __float_as_uint(__fsub_rn(dd, m));
    z = __float_as_uint(__fsub_rn(0.5f, dd));
}

// RULE: 0 RNG (NSG, HNSW layers), 1 tau-MNG, 2 alpha-PG (angles up to 60
// degrees; wider angles stay on the FP32 prune, whose per-pair angle test the
// screen above cannot skip: evaluated on every near pair of the triangle it
// made the tile version ten times slower than RNG, 3.9 s against 0.37 s per
// 2M-row build).
template <int RULE>
__global__ void __launch_bounds__(PG_THREADS, 1) prune_gram_kernel(PgArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t tiles_s = (smem_u32(smem_raw) + 1023u) & ~1023u; // swizzled tiles need 1024-byte alignment
    unsigned char *tiles = smem_raw + (tiles_s - smem_u32(smem_raw));
    PgShared &S = *reinterpret_cast<PgShared *>(tiles + NSLOT * CHUNK_BYTES);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkb = ((int)a.ld + 63) >> 6;

    // K padding beyond ld is never written by the loaders and must read as zero
    for (int i = tid; i < (int)(NSLOT * CHUNK_BYTES / 16); i += PG_THREADS)
        reinterpret_cast<uint4 *>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 1) tmem_alloc(&S.tmem, NACC * PC);
    if (tid == 0) {
        for (int i = 0; i < NSLOT; ++i) {
            mbar_init(&S.slot_full[i], NLOAD * 32); // every loader lane, after its copies and a proxy fence
            mbar_init(&S.slot_empty[i], 1);         // MMA commit after the chunk's last tile
        }
        for (int i = 0; i < NACC; ++i) {
            mbar_init(&S.acc_full[i], 1);   // MMA commit
            mbar_init(&S.acc_empty[i], EPI);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&S.keys_full[i], 1);        // metadata lane 0 (expect_tx); the bulk copy completes it
            mbar_init(&S.ids_ready[i], 1);        // metadata lane 0 after the keys are parsed
            mbar_init(&S.meta_full[i], 64);       // metadata lanes: stores done, norm copies landed
            mbar_init(&S.bound_ready[i], EPI);    // mask builders' shares of the RNG column values
            mbar_init(&S.mask_full[i], EPI);
            mbar_init(&S.node_empty[i], 2 + NLOAD); // scan, MMA issuer, loader warps
        }
        S.abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t slot0 = tiles_s;
    bool ok = true;

    if (warp == 0) {
        // ------------------------------------------------------------ metadata
        // node kk's pool prefix (the candidates and the entry before them) by
        // one bulk copy from an even pool index; lane 0 issues
        uint32_t r_cnt0 = 0u, r_cnt1 = 0u, r_shift0 = 0u, r_shift1 = 0u;
        int pending = -1; // node whose key copy is requested and not yet waited for
        auto request = [&](int kk) {
            const uint32_t q = blockIdx.x + (uint32_t)kk * gridDim.x; // item: node, or staged list
            if (q >= a.n_items) return;
            const int b = kk & 1;
            pending = kk;
            const uint32_t row = a.by_node ? a.nodes[q] : q;
            const uint32_t cnt = min(a.pool_cnt[row], a.cap);
            const uint64_t base = (uint64_t)row * a.cap;
            const uint32_t shift = (uint32_t)(base & 1u);
            const uint32_t ncopy = min(cnt, (uint32_t)max(a.maxc, 2));
            const uint32_t nent = (shift + ncopy + 1u) & ~1u;
            if (b) {
                r_cnt1 = cnt;
                r_shift1 = shift;
            } else {
                r_cnt0 = cnt;
                r_shift0 = shift;
            }
            if (lane == 0) {
                if (nent) {
                    fence_proxy_async(); // earlier generic reads of the buffer before the async-proxy write
                    mbar_arrive_expect_tx(&S.keys_full[b], nent * 8u);
                    bulk_copy_g2s(smem_u32(S.meta[b].key), a.pool + (base - shift), nent * 8u, &S.keys_full[b]);
                } else {
                    mbar_arrive(&S.keys_full[b]);
                }
            }
        };
        request(0);
        int k = 0;
        for (uint32_t q = blockIdx.x; q < a.n_items; q += gridDim.x, ++k) {
            const int sl = k & 1;
            if (!mbar_wait(&S.keys_full[sl], (k >> 1) & 1)) { ok = false; break; }
            pending = -1;
            if (S.abort_flag) { ok = false; break; }
            NodeMeta &M = S.meta[sl];
            const int cnt = (int)(sl ? r_cnt1 : r_cnt0);
            const uint32_t shift = sl ? r_shift1 : r_shift0;
            const uint32_t node = a.nodes ? a.nodes[q] : q;
            int first = 0;
            if (cnt > 0 && kcna_key_id(M.key[shift]) == node) first = 1;
            const int nc = first < cnt ? max(min(cnt, a.maxc), first + 1) - first : 0;
            const int nch = (nc + PC - 1) / PC;
            const uint32_t koff = shift + (uint32_t)first;
#pragma unroll 4
            for (int i = 0; i < MW; ++i) {
                const int c = 32 * i + lane;
                const bool live = c < nc;
                uint32_t id = 0u, before = 0xFFFFFFFFu;
                float pd = 0.f;
                if (live) {
                    const uint64_t key = M.key[koff + c];
                    id = kcna_key_id(key);
                    pd = kcna_key_dist(key);
                    if (c > 0) before = kcna_key_id(M.key[koff + c - 1]);
                }
                // src/kgraph.cpp:1822: ids beyond the layer prefix are skipped; a
                // repeated id is occluded by its twin (same row, same distance)
                const bool dead = !live || (c > 0 && (id >= a.N || id == before));
                const unsigned dm = __ballot_sync(KCNA_FULL, dead);
                if (c < nch * PC) {
                    M.pd[c] = pd;
                    if (live && id < a.N) cp_async4(smem_u32(&M.nrm[c]), a.norms + id);
                    else M.nrm[c] = 0.f;
                }
                if (lane == 0) M.dead[i] = dm;
            }
            if (lane == 0) {
                M.q = node;
                M.nc = (uint32_t)nc;
                M.nch = (uint32_t)nch;
                M.koff = koff;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.ids_ready[sl]);
            mbar_arrive_cp_async(&S.meta_full[sl]); // when this lane's norm copies have landed
            mbar_arrive(&S.meta_full[sl]);          // this lane's stores
            // the next node's keys into the other buffer, once its node k-1 is done
            const uint32_t qn = q + gridDim.x;
            if (qn < a.n_items) {
                if (k >= 1 && !mbar_wait(&S.node_empty[sl ^ 1], ((k - 1) >> 1) & 1)) { ok = false; break; }
                request(k + 1);
            }
        }
        cp_async_wait_0();
        // a key copy still in flight lands before the block exits
        if (pending >= 0) (void)mbar_wait(&S.keys_full[pending & 1], (pending >> 1) & 1, 1u << 16);
        if (!ok) S.abort_flag = 1;
    } else if (warp >= LOAD_WARP) {
        // --------------------------------------------------------- row loaders
        const int lw = warp - LOAD_WARP;
        const int nseg = (int)(a.ld >> 3); // 16-byte segments per row
        uint32_t gc = 0;
        int pend = -1; // slot whose copies are in flight, not yet announced
        int k = 0;
        for (uint32_t q = blockIdx.x; q < a.n_items; q += gridDim.x, ++k) {
            const int sl = k & 1;
            if (!mbar_wait(&S.ids_ready[sl], (k >> 1) & 1) || S.abort_flag) { ok = false; break; }
            const NodeMeta &M = S.meta[sl];
            const int nc = (int)M.nc, nch = (int)M.nch;
            const uint64_t *keys = M.key + M.koff;
            for (int i = 0; i < nch; ++i, ++gc) {
                const int s = (int)(gc % NSLOT);
                if (gc >= (uint32_t)NSLOT && !mbar_wait(&S.slot_empty[s], ((gc / NSLOT) - 1) & 1)) {
                    ok = false;
                    break;
                }
                const uint32_t slot = slot0 + (uint32_t)s * CHUNK_BYTES;
                const int seg = lane & 15;
#pragma unroll 4
                for (int rr = 0; rr < 16; ++rr) {
                    const int r = 32 * lw + 2 * rr + (lane >> 4); // row of the chunk
                    const int c = PC * i + r;
                    if (c < nc && seg < nseg) {
                        const uint32_t id = kcna_key_id(keys[c]);
                        cp_async16(slot + (uint32_t)(seg >> 3) * PC * KBB + sw128_off((uint32_t)r, (uint32_t)(seg & 7)),
                                   a.rows + (uint64_t)id * a.ld + seg * 8);
                    }
                }
                cp_async_commit();
                if (pend >= 0) { // the previous chunk's copies: landed, fenced for the tensor cores, announced
                    cp_async_wait_1();
                    fence_proxy_async();
                    mbar_arrive(&S.slot_full[pend]);
                }
                pend = s;
            }
            if (pend >= 0) {
                cp_async_wait_0();
                fence_proxy_async();
                mbar_arrive(&S.slot_full[pend]);
                pend = -1;
            }
            if (!ok) break;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.node_empty[sl]);
        }
        cp_async_wait_0();
        if (!ok) S.abort_flag = 1;
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            uint32_t gc = 0, acount = 0;
            int k = 0;
            const uint32_t idesc = idesc_bf16(PC, PC);
            for (uint32_t q = blockIdx.x; q < a.n_items && ok; q += gridDim.x, ++k) {
                const int sl = k & 1;
                if (!mbar_wait(&S.ids_ready[sl], (k >> 1) & 1) || S.abort_flag) { ok = false; break; }
                const int nch = (int)S.meta[sl].nch;
                for (int J = 0; J < nch && ok; ++J)
                    for (int I = J; I < nch; ++I, ++acount) {
                        const uint32_t gI = gc + (uint32_t)I, gJ = gc + (uint32_t)J;
                        if (J == 0 && !mbar_wait(&S.slot_full[gI % NSLOT], (gI / NSLOT) & 1)) { ok = false; break; }
                        const int b = (int)(acount % NACC);
                        if (acount >= (uint32_t)NACC && !mbar_wait(&S.acc_empty[b], ((acount / NACC) - 1) & 1)) {
                            ok = false;
                            break;
                        }
                        fence_after();
                        const uint32_t aJ = slot0 + (gJ % NSLOT) * CHUNK_BYTES, bI = slot0 + (gI % NSLOT) * CHUNK_BYTES;
                        for (int kb = 0; kb < nkb; ++kb)
#pragma unroll
                            for (int kk = 0; kk < 4; ++kk)
                                mma_bf16(tmem + (uint32_t)(b * PC), desc_sw128(aJ + kb * PC * KBB + kk * 32),
                                         desc_sw128(bI + kb * PC * KBB + kk * 32), idesc, (kb | kk) ? 1u : 0u);
                        mma_commit(&S.acc_full[b]);
                        if (I == nch - 1) mma_commit(&S.slot_empty[gJ % NSLOT]); // chunk J's last tile
                    }
                gc += (uint32_t)nch;
                if (ok) mbar_arrive(&S.node_empty[sl]); // this node's tiles are issued
            }
            if (!ok) {
                S.abort_flag = 1;
                // products still in flight finish before TMEM is released
                for (uint32_t b = 0; b < (uint32_t)NACC; ++b)
                    if (acount > b) {
                        const uint32_t last = b + (acount - 1 - b) / NACC * NACC;
                        (void)mbar_wait(&S.acc_full[b], (last / NACC) & 1u, 1u << 16);
                    }
            }
        }
        __syncwarp();
    } else if (warp < SCAN_WARP) {
        // -------------------------------------------------------- mask builders
        const int qt = warp & 3, h = (warp - 2) >> 2; // TMEM lane quarter, column group
        uint32_t acount = 0;
        int k = 0;
        for (uint32_t q = blockIdx.x; q < a.n_items; q += gridDim.x, ++k) {
            const int sl = k & 1;
            bool mine = mbar_wait(&S.meta_full[sl], (k >> 1) & 1) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            NodeMeta &M = S.meta[sl];
            uint32_t *mask = S.mask[sl];
            const int nch = (int)M.nch;
            if (RULE == 0) { // column values pd - |p|^2 in place of pd (the scan reads distances from the keys)
                for (int c = (warp - 2) * 32 + lane; c < nch * PC; c += EPI * 32)
                    M.pd[c] = __fsub_rn(M.pd[c], M.nrm[c]);
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.bound_ready[sl]);
                mine = mbar_wait(&S.bound_ready[sl], (k >> 1) & 1);
                if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            }
            for (int J = 0; J < nch && ok; ++J) {
                const int t = J * PC + 32 * qt + lane; // occluder candidate (TMEM lane)
                const float n_t = M.nrm[t], td = M.pd[t];
                const uint32_t id_t = RULE == 2 ? kcna_key_id(M.key[M.koff + t]) : 0u;
                const float k2 = 2.f - a.aux, ctd = -16.f - td; // alpha-PG screen (alpha_signs)
                for (int I = J; I < nch; ++I, ++acount) {
                    const int b = (int)(acount % NACC);
                    mine = mbar_wait(&S.acc_full[b], (acount / NACC) & 1);
                    fence_after();
                    const bool skip = I == J && CW * h + CW - 1 <= 32 * qt; // no column after any row of the warp
                    uint32_t raw[CW];
                    if (mine && !skip) {
                        const uint32_t ta = tmem + ((uint32_t)(32 * qt) << 16) + (uint32_t)(b * PC + CW * h);
#pragma unroll
                        for (int x = 0; x < CW / 16; ++x) tmem_ld16_async(ta + 16 * x, raw + 16 * x);
#pragma unroll
                        for (int x = 0; x < CW / 16; ++x) tmem_wait_ld16(raw + 16 * x);
                    }
                    // the accumulator is in registers: release it before the bit work
                    fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.acc_empty[b]);
                    if (!__all_sync(KCNA_FULL, mine)) {
                        ok = false;
                        break;
                    }
#pragma unroll
                    for (int ww = 0; ww < WPT; ++ww) {
                        const int p0 = I * PC + CW * h + 32 * ww; // first candidate of the word
                        uint32_t word = 0;
                        if (!skip) {
                            const float4 *np4 = reinterpret_cast<const float4 *>(M.nrm + p0);
                            const float4 *pd4 = reinterpret_cast<const float4 *>(M.pd + p0);
                            // four chains of eight: candidate 8j+m ends in bit 7-m of wq[j]
                            uint32_t wq[4] = {0u, 0u, 0u, 0u};
                            uint32_t wo[4] = {0u, 0u, 0u, 0u}, wz[4] = {0u, 0u, 0u, 0u}; // alpha-PG
#pragma unroll
                            for (int u4 = 0; u4 < 8; ++u4) {
                                const float4 n4 = np4[u4], d4 = pd4[u4];
                                const float nn[4] = {n4.x, n4.y, n4.z, n4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
                                for (int v = 0; v < 4; ++v) {
                                    const float g = __uint_as_float(raw[32 * ww + 4 * u4 + v]);
                                    if (RULE == 2) {
                                        uint32_t r, o, z;
                                        alpha_signs(g, n_t, nn[v], dv[v], k2, ctd, r, o, z);
                                        wq[u4 >> 1] = __funnelshift_l(r, wq[u4 >> 1], 1);
                                        wo[u4 >> 1] = __funnelshift_l(o, wo[u4 >> 1], 1);
                                        wz[u4 >> 1] = __funnelshift_l(z, wz[u4 >> 1], 1);
                                    } else {
                                        const uint32_t sg = occl_sign<RULE>(g, n_t, nn[v], dv[v], a.aux);
                                        wq[u4 >> 1] = __funnelshift_l(sg, wq[u4 >> 1], 1); // shifts the sign bit in
                                    }
                                }
                            }
                            word = __brev((wq[0] << 24) | (wq[1] << 16) | (wq[2] << 8) | wq[3]);
                            uint32_t amb = 0u; // alpha-PG: pairs left to the exact angle test (bit = candidate - p0)
                            if (RULE == 2) {
                                const uint32_t occ = __brev((wo[0] << 24) | (wo[1] << 16) | (wo[2] << 8) | wo[3]) &
                                                     __brev((wz[0] << 24) | (wz[1] << 16) | (wz[2] << 8) | wz[3]);
                                amb = word & ~occ;
                                word = occ;
                            }
                            if (I == J) { // only candidates after t
                                const int r = t - p0;
                                const uint32_t after = r < 0 ? 0xFFFFFFFFu : r >= 31 ? 0u : ~((2u << r) - 1u);
                                word &= after;
                                amb &= after;
                            }
                            if (RULE == 2) { // near-equilateral pairs and zero sides: the exact test (rare)
                                // only between candidates of this node: rows and columns beyond nc hold
                                // stale keys (their bits are never read by the scan)
                                const int nv = (int)M.nc - p0;
                                amb &= t >= (int)M.nc || nv <= 0 ? 0u : nv >= 32 ? 0xFFFFFFFFu : (1u << nv) - 1u;
                                while (amb) {
                                    const int v = __ffs(amb) - 1;
                                    amb &= amb - 1u;
                                    const uint32_t id_p = kcna_key_id(M.key[M.koff + p0 + v]);
                                    if (id_t >= a.N || id_p >= a.N) continue; // beyond the layer prefix: dead
                                    const float djk = rows_l2(RowsB16{a.rows, (int)a.ld}, id_t, id_p);
                                    if (alpha_angle_exact(td, djk, M.pd[p0 + v], a.thr)) word |= 1u << v;
                                }
                            }
                        }
                        mask[mask_base(4 * I + CW / 32 * h + ww) + t] = word;
                    }
                }
            }
            if (!ok) break;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.mask_full[sl]);
        }
        if (!ok) S.abort_flag = 1;
    } else {
        // ----------------------------------------------------------------- scan
        unsigned long long cc = 0;
        int k = 0;
        for (uint32_t q = blockIdx.x; q < a.n_items; q += gridDim.x, ++k) {
            const int sl = k & 1;
            const bool mine = mbar_wait(&S.mask_full[sl], (k >> 1) & 1) && !S.abort_flag;
            if (!__all_sync(KCNA_FULL, mine)) { ok = false; break; }
            const NodeMeta &M = S.meta[sl];
            const uint32_t *mask = S.mask[sl];
            const uint64_t *keys = M.key + M.koff;
            const int nc = (int)M.nc;
            uint32_t *gi = a.g_ids + (uint64_t)M.q * a.W;
            float *gd = a.g_dist + (uint64_t)M.q * a.W;
            int nk = 0;
            if (nc > 0) {
                uint32_t dead = lane < MW ? M.dead[lane] : 0xFFFFFFFFu;
                int t = 0;
                for (;;) {
                    if (lane == 0) {
                        gi[nk] = kcna_key_id(keys[t]);
                        gd[nk] = kcna_key_dist(keys[t]);
                        cc += (unsigned long long)nk; // a kept candidate was tested against every earlier one
                    }
                    ++nk;
                    if (nk >= a.range) break;
                    const int tw = t >> 5;
                    uint32_t o = 0;
                    if (lane < MW && lane >= 4 * (t >> 7)) o = mask[mask_base(lane) + t];
                    const uint32_t above = lane > tw ? 0xFFFFFFFFu : lane < tw ? 0u : ~((2u << (t & 31)) - 1u);
                    cc += (unsigned long long)nk * __popc(o & ~dead & above); // dropped at the nk-th kept
                    dead |= o;
                    const uint32_t alive = ~dead & above;
                    const unsigned bal = __ballot_sync(KCNA_FULL, alive != 0u);
                    if (!bal) break;
                    const int L = __ffs(bal) - 1;
                    t = 32 * L + __ffs(__shfl_sync(KCNA_FULL, alive, L)) - 1;
                }
            }
            __syncwarp();
            for (int j = nk + lane; j < (int)a.W; j += 32) {
                gi[j] = KCNA_NONE;
                gd[j] = 0.f;
            }
            if (lane == 0) a.g_deg[M.q] = (uint32_t)nk;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.node_empty[sl]);
        }
        cc = kcna_warp_sum(cc);
        if (lane == 0 && cc) atomicAdd(a.comps, cc);
        if (!ok) S.abort_flag = 1;
    }
    fence_before();
    __syncthreads();
    if (warp == 1) tmem_free(tmem, NACC * PC);
    if (!ok) kcna_set_err(a.err, KCNA_DERR_SPIN);
}

size_t prune_gram_smem() { return 1024 + (size_t)NSLOT * CHUNK_BYTES + sizeof(PgShared); }

template <int RULE>
kcna_status launch_rule(kcna_ctx *c, const PgArgs &a, uint32_t grid) {
    const size_t sm = prune_gram_smem();
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(prune_gram_kernel<RULE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm),
                             "prune_gram smem attr"));
    prune_gram_kernel<RULE><<<grid, PG_THREADS, sm, c->stream>>>(a);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "prune_gram_kernel");
}

} // namespace

bool kcna_prune_tc_ok(const kcna_ctx *c, int kind, int range, int maxc, float angle) {
    // alpha-PG: the angle screen proves the test for thresholds cos(angle) >= cos(60 degrees)
    if (kind == KCNA_ALPHAPG && !(kcna_alpha_threshold(angle) >= kcna_alpha_threshold(60.f))) return false;
    return c->gram_exact && c->Xh && c->norms && !(c->ld & 7u) && c->ld <= 128 && range >= 1 && maxc >= 1 &&
           maxc <= MAXC && prune_gram_smem() <= 227 * 1024;
}

kcna_status kcna_prune_tc_launch(kcna_ctx *c, int kind, float t3, float angle, int range, int maxc,
                                 unsigned long long *comps, const uint64_t *keys, uint64_t stride, const uint32_t *cnt,
                                 const uint32_t *nodes, uint32_t n_items, bool pool_list) {
    if (!kcna_prune_tc_ok(c, kind, range, maxc, angle))
        return kcna_fail(c, KCNA_E_STATE, "Gram-tile prune needs Gram-exact rows");
    if (pool_list && !nodes) return kcna_fail(c, KCNA_E_ARG, "Gram-tile prune: pool-list mode needs a node list");
    const bool staged = nodes && !pool_list;
    PgArgs a;
    a.N = staged ? 0xFFFFFFFFu : c->n; // staged lists carry no layer prefix
    a.cap = staged ? (uint32_t)stride : c->cap;
    a.n_items = nodes ? n_items : c->n;
    a.nodes = nodes;
    a.by_node = pool_list ? 1u : 0u;
    a.W = c->W;
    a.ld = c->ld;
    a.pool = staged ? keys : c->pool;
    a.rows = c->Xh;
    a.pool_cnt = staged ? cnt : c->pool_cnt;
    a.norms = c->norms;
    a.thr = kcna_alpha_threshold(angle);
    // tau-MNG: 3 tau; alpha-PG: 4m, m = 1/2 - thr + 1e-5 (the angle screen's margin)
    a.aux = kind == KCNA_TAUMNG ? t3 : kind == KCNA_ALPHAPG ? (float)(4.0 * (0.5 - (double)a.thr + 1e-5)) : 0.f;
    a.range = range;
    a.maxc = maxc;
    a.g_ids = c->g_ids;
    a.g_dist = c->g_dist;
    a.g_deg = c->g_deg;
    a.comps = comps;
    a.err = c->d_err;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(a.n_items, (uint64_t)std::max(c->num_sms, 1));
    if (grid == 0) return KCNA_OK;
    if (kind == KCNA_TAUMNG) return launch_rule<1>(c, a, grid);
    if (kind == KCNA_ALPHAPG) return launch_rule<2>(c, a, grid);
    return launch_rule<0>(c, a, grid);
}
