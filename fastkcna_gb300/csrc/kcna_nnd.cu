// kcna_nnd.cu - NN-descent on device-resident pools.
//
// Replaces the KGraphConstructor constructor loop (src/kgraph.cpp:1281-1459):
// init (:1001-1044), join (:1097-1117 with Nhood::join :970-987 and
// parallel_try_insert :948-967), update (:1118-1202) and the per-iteration
// statistics / stop rule (:1365-1426).
//
// GPU form of one iteration:
//   join    one block per node n: gather the node's new list A and old list B,
//           compute every pair of A x A (i < j) and A x B with the canonical
//           FMA-chain distance in register tiles (rows staged through shared
//           memory in 32-float chunks), and emit each pair to both endpoints'
//           candidate buffers when it is within that endpoint's radius.
//           Candidates of one target from one block are written as one
//           contiguous run after a single atomicAdd.
//   merge   one block per node: sort the candidate buffer, drop duplicates,
//           merge with the sorted pool by rank, keep the best `limit`; new
//           entries carry flag=new (the reference's InsertIntoPool
//           :261-298 semantics applied to a batch).
//   sample  the update step: M (prefix holding S new entries), radiusM, the
//           forward new/old lists and reverse lists (atomics, capped buffers,
//           random subset of R chosen in the join).
// The reference inserts into locked pools while joining, so its result depends
// on thread timing; this batched form inserts all of an iteration's
// candidates at its end.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>

#include "kcna_internal.h"
#include "kcna_join.cuh"
#include "kcna_sort.cuh"

namespace {

// ---------------------------------------------------------------------------
// init: S random pool entries + 2S random ids as the first new list.
// GenRandom (src/kgraph.cpp:82-110): size values < N-size, sorted, made
// strictly increasing, shifted by a random offset mod N.  Done per warp with a
// bitonic sort and a prefix maximum (a[i] = i + max_{j<=i}(a[j]-j)).
// ---------------------------------------------------------------------------
__device__ void warp_gen_random(uint64_t seed, uint64_t stream, uint32_t size, uint32_t N, uint32_t *s_out,
                                uint64_t *s_tmp) {
    const int lane = kcna_lane();
    if (N == size) {
        for (uint32_t i = lane; i < size; i += 32) s_out[i] = i;
        __syncwarp();
        return;
    }
    int p = kcna_pow2_ceil_d((int)size);
    for (int i = lane; i < p; i += 32)
        s_tmp[i] = i < (int)size ? (uint64_t)(kcna_rand32(seed, stream, i) % (N - size)) : KCNA_EMPTY_KEY;
    kcna_warp_bitonic(s_tmp, p);
    // prefix max of a[j]-j over j, chunk by chunk of 32
    int64_t carry = INT64_MIN;
    for (uint32_t base = 0; base < size; base += 32) {
        uint32_t i = base + lane;
        int64_t v = i < size ? (int64_t)s_tmp[i] - (int64_t)i : INT64_MIN;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t u = __shfl_up_sync(KCNA_FULL, v, o);
            if (lane >= o && u > v) v = u;
        }
        if (carry > v) v = carry;
        carry = __shfl_sync(KCNA_FULL, v, 31);
        if (i < size) s_out[i] = (uint32_t)((int64_t)i + v);
    }
    __syncwarp();
    uint32_t off = kcna_rand32(seed, stream, 0xFFFFFFull) % N;
    for (uint32_t i = lane; i < size; i += 32) s_out[i] = (uint32_t)(((uint64_t)s_out[i] + off) % N);
    __syncwarp();
}

__global__ void __launch_bounds__(128) init_kernel(const float *__restrict__ X, int ld, uint32_t N, uint32_t S,
                                                   uint32_t cap, uint64_t seed, uint64_t *__restrict__ pool,
                                                   uint32_t *__restrict__ pool_cnt,
                                                   uint32_t *__restrict__ fwd_new, uint32_t fwd_new_cap,
                                                   uint32_t *__restrict__ fwd_new_cnt) {
    __shared__ uint32_t s_ids[4][128];
    __shared__ uint64_t s_tmp[4][128];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    const uint32_t n = blockIdx.x * 4 + w;
    if (n >= N) return;
    // first new list: 2S random ids (may include n itself, as in the reference)
    warp_gen_random(seed, (uint64_t)n * 4 + 0, 2 * S, N, s_ids[w], s_tmp[w]);
    for (uint32_t i = lane; i < 2 * S; i += 32) fwd_new[(uint64_t)n * fwd_new_cap + i] = s_ids[w][i];
    if (lane == 0) fwd_new_cnt[n] = 2 * S;
    __syncwarp();
    // pool: S+1 random ids, n dropped, first S kept
    warp_gen_random(seed, (uint64_t)n * 4 + 1, S + 1, N, s_ids[w], s_tmp[w]);
    uint64_t key = KCNA_EMPTY_KEY;
    {
        uint32_t r = lane <= (int)S ? s_ids[w][lane] : n;
        bool keep = lane <= (int)S && r != n;
        unsigned mk = __ballot_sync(KCNA_FULL, keep);
        int pos = __popc(mk & kcna_lanemask_lt());
        if (keep && pos < (int)S) {
            float dd = kcna_l2_ldg(X + (uint64_t)r * ld, X + (uint64_t)n * ld, ld);
            key = kcna_key(dd, r, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
        }
    }
    key = kcna_warp_sort32(key);
    uint64_t *pr = pool + (uint64_t)n * cap;
    for (uint32_t i = lane; i < cap; i += 32) pr[i] = (i == (uint32_t)lane && i < S) ? key : KCNA_EMPTY_KEY;
    if (lane == 0) pool_cnt[n] = S;
}

// ---------------------------------------------------------------------------
// join
// ---------------------------------------------------------------------------
constexpr int JT = 256;      // threads per join block
constexpr int JCOLS = 64;    // columns per tile chunk
constexpr int JKC = 32;      // floats per k chunk
constexpr int JKP = JKC + 4; // padded row pitch in shared memory

template <int RI, class R> // rows per thread = RI, tile rows = 32 * RI
__device__ void join_tiles(const JoinArgs &a, const R &rows, uint32_t node, const uint32_t *s_A, int na, const uint32_t *s_B, int nb,
                           float *s_As, float *s_Bs, float *s_D, const float *s_radA, unsigned *s_emit) {
    constexpr int RA = 32 * RI;
    const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3; // 8 col groups x 32 row groups
    const int ncol = na + nb;
    const int ld = a.ld;
    for (int c0 = 0; c0 < ncol; c0 += JCOLS) {
        // rows that can pair with this chunk: i < min(na, c0+JCOLS) (i < j inside A)
        const int rows_needed = min(na, c0 + JCOLS);
        float acc[RI][8];
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
        for (int k0 = 0; k0 < ld; k0 += JKC) {
            // stage A rows (RA x 32 floats) and chunk columns (64 x 32 floats)
            for (int idx = tid; idx < RA * (JKC / 4); idx += JT) {
                int r = idx >> 3, c = (idx & 7) * 4;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r < rows_needed && k0 + c < ld) v = rows.ld4(s_A[r], (k0 + c) >> 2);
                *reinterpret_cast<float4 *>(s_As + r * JKP + c) = v;
            }
            for (int idx = tid; idx < JCOLS * (JKC / 4); idx += JT) {
                int r = idx >> 3, c = (idx & 7) * 4;
                int col = c0 + r;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (col < ncol && k0 + c < ld) {
                    uint32_t id = col < na ? s_A[col] : s_B[col - na];
                    v = rows.ld4(id, (k0 + c) >> 2);
                }
                *reinterpret_cast<float4 *>(s_Bs + r * JKP + c) = v;
            }
            __syncthreads();
            const int kend = min(JKC, ld - k0);
            for (int k = 0; k < kend; k += 4) {
                float4 ra[RI], cb[8];
#pragma unroll
                for (int i = 0; i < RI; ++i) ra[i] = *reinterpret_cast<const float4 *>(s_As + (ty + 32 * i) * JKP + k);
#pragma unroll
                for (int j = 0; j < 8; ++j) cb[j] = *reinterpret_cast<const float4 *>(s_Bs + (tx + 8 * j) * JKP + k);
#pragma unroll
                for (int i = 0; i < RI; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = kcna_acc4(acc[i][j], ra[i], cb[j]);
            }
            __syncthreads();
        }
        // distances of the chunk to shared memory: s_D[row][col], pitch JCOLS+1
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) s_D[(ty + 32 * i) * (JCOLS + 1) + tx + 8 * j] = acc[i][j];
        __syncthreads();
        // emission: warp w handles row targets, then column targets
        const int warp = tid >> 5, lane = tid & 31, nwarp = JT / 32;
        const int cend = min(JCOLS, ncol - c0);
        // row targets: A[i] receives column ids
        for (int i = warp; i < rows_needed; i += nwarp) {
            uint32_t tgt = s_A[i];
            float rad = s_radA[i];
            int cnt = 0;
            uint64_t keys[2];
            bool ok[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int cl = lane + 32 * h, col = c0 + cl;
                ok[h] = false;
                if (cl < cend && (col >= na || i < col)) {
                    uint32_t id = col < na ? s_A[col] : s_B[col - na];
                    float dd = s_D[i * (JCOLS + 1) + cl];
                    if (id != tgt && dd <= rad) {
                        ok[h] = true;
                        keys[h] = kcna_key(dd, id, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
                    }
                }
            }
            unsigned m0 = __ballot_sync(KCNA_FULL, ok[0]), m1 = __ballot_sync(KCNA_FULL, ok[1]);
            cnt = __popc(m0) + __popc(m1);
            if (cnt == 0) continue;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(a.cand_cnt + tgt, (uint32_t)cnt);
            base = __shfl_sync(KCNA_FULL, base, 0);
            const uint64_t s0 = (uint64_t)tgt * a.CB;
            if (ok[0]) {
                uint32_t p = base + __popc(m0 & kcna_lanemask_lt());
                if (p < a.CB) kcna_cand_put(a.cand, s0 + p, keys[0], node);
            }
            if (ok[1]) {
                uint32_t p = base + __popc(m0) + __popc(m1 & kcna_lanemask_lt());
                if (p < a.CB) kcna_cand_put(a.cand, s0 + p, keys[1], node);
            }
            if (lane == 0) atomicAdd(s_emit, (unsigned)cnt);
        }
        // column targets: column id receives row ids
        for (int cl = warp; cl < cend; cl += nwarp) {
            int col = c0 + cl;
            uint32_t tgt = col < na ? s_A[col] : s_B[col - na];
            float rad = __ldg(a.radius + tgt);
            unsigned mk[RI];
            uint64_t keys[RI];
            int cnt = 0;
#pragma unroll
            for (int h = 0; h < RI; ++h) {
                int i = lane + 32 * h;
                bool ok = false;
                if (i < rows_needed && (col >= na || i < col)) {
                    uint32_t id = s_A[i];
                    float dd = s_D[i * (JCOLS + 1) + cl];
                    if (id != tgt && dd <= rad) {
                        ok = true;
                        keys[h] = kcna_key(dd, id, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
                    }
                }
                mk[h] = __ballot_sync(KCNA_FULL, ok);
                cnt += __popc(mk[h]);
            }
            if (cnt == 0) continue;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(a.cand_cnt + tgt, (uint32_t)cnt);
            base = __shfl_sync(KCNA_FULL, base, 0);
            const uint64_t s0 = (uint64_t)tgt * a.CB;
            uint32_t run = base;
#pragma unroll
            for (int h = 0; h < RI; ++h) {
                if (mk[h] & (1u << lane)) {
                    uint32_t p = run + __popc(mk[h] & kcna_lanemask_lt());
                    if (p < a.CB) kcna_cand_put(a.cand, s0 + p, keys[h], node);
                }
                run += __popc(mk[h]);
            }
            if (lane == 0) atomicAdd(s_emit, (unsigned)cnt);
        }
        __syncthreads();
    }
}

template <class R>
__global__ void __launch_bounds__(JT, 3) join_kernel(JoinArgs a, R rows) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *s_As = reinterpret_cast<float *>(smem);                // 128 x JKP
    float *s_Bs = s_As + 128 * JKP;                               // JCOLS x JKP
    float *s_D = s_Bs + JCOLS * JKP;                              // 128 x (JCOLS+1)
    float *s_radA = s_D + 128 * (JCOLS + 1);                      // capA
    uint32_t *s_A = reinterpret_cast<uint32_t *>(s_radA + a.capA); // capA
    uint32_t *s_B = s_A + a.capA;                                 // capB
    __shared__ unsigned s_emit;
    const uint32_t node = blockIdx.x;
    // new list: forward new then a random subset (<= R) of reverse new
    uint32_t fn = min(a.fwd_new_cnt[node], a.fwd_new_cap);
    for (uint32_t i = threadIdx.x; i < fn; i += blockDim.x) s_A[i] = a.fwd_new[(uint64_t)node * a.fwd_new_cap + i];
    uint32_t fo = min(a.fwd_old_cnt[node], a.fwd_old_cap);
    for (uint32_t i = threadIdx.x; i < fo; i += blockDim.x) s_B[i] = a.fwd_old[(uint64_t)node * a.fwd_old_cap + i];
    __syncthreads();
    uint32_t rn = 0, ro = 0;
    if (a.iter > 0) {
        rn = take_reverse(a.rnew + (uint64_t)node * a.RB, a.rnew_cnt[node], a.R, s_A + fn);
        ro = take_reverse(a.rold + (uint64_t)node * a.RB, a.rold_cnt[node], a.R, s_B + fo);
        __syncthreads();
    }
    // at most 128 rows per tile; the forward list alone is <= S + R < 128 in practice
    const int na = (int)min(fn + rn, 128u), nb = (int)(fo + ro);
    for (int i = threadIdx.x; i < na; i += blockDim.x) s_radA[i] = __ldg(a.radius + s_A[i]);
    __syncthreads();
    if (na == 0) return;
    if (threadIdx.x == 0) {
        atomicAdd(a.counters + 0, (unsigned long long)((uint64_t)na * (na - 1) / 2 + (uint64_t)na * nb));
        atomicAdd(a.counters + 5, (unsigned long long)(na + nb));
        s_emit = 0;
    }
    if (na <= 32)
        join_tiles<1>(a, rows, node, s_A, na, s_B, nb, s_As, s_Bs, s_D, s_radA, &s_emit);
    else if (na <= 64)
        join_tiles<2>(a, rows, node, s_A, na, s_B, nb, s_As, s_Bs, s_D, s_radA, &s_emit);
    else
        join_tiles<4>(a, rows, node, s_A, na, s_B, nb, s_As, s_Bs, s_D, s_radA, &s_emit);
    if (threadIdx.x == 0 && s_emit) atomicAdd(a.counters + 6, (unsigned long long)s_emit);
}

// ---------------------------------------------------------------------------
// merge: candidates of one node into its pool (batched InsertIntoPool)
// ---------------------------------------------------------------------------
constexpr int MT = 256;

struct MergeArgs {
    uint64_t *pool;
    uint32_t *pool_cnt;
    uint32_t cap, limit, K;
    float *radius;
    uint64_t *cand; // key and joiner per slot (kcna_cand_put)
    uint32_t *cand_cnt;
    uint32_t CB;
    unsigned long long *counters; // [1] flagged in top-K, [2] overflow, [3] inserted
    // found credit (NN-descent merges): the joiner of every candidate, and the
    // flags the merge sets.  The reference's join marks a node found when one
    // of the pairs its join evaluated was inserted below K by its
    // parallel_try_insert (src/kgraph.cpp:1107-1116); a pair several joiners
    // evaluate is inserted by the first to reach the pool, and only that one
    // is credited.  Here each distinct new entry placed at rank < K credits the
    // lowest joiner that emitted it (in the reference's increasing-node
    // parallel loop, in practice the first to reach the pair).  Crediting every
    // emitter instead over-credits: NN-descent then converges measurably
    // faster than the reference's (200k C2 rows: recall 0.9968 after six
    // iterations against the reference's 0.9943).
    uint32_t credit; // credit joiners (NN-descent merges)
    uint8_t *found;
    uint32_t n_nodes;
};

// Warp-per-node merge, survivors first.  Every candidate is looked up in the
// node's sorted pool by binary search (shared memory): a candidate equal to a
// pool entry, or one that would land at rank >= limit, is dropped.  In a
// converging NN-descent almost every candidate is such a repeat, so only the
// few survivors are sorted, deduplicated and merged, and only the pool entries
// they displace are written.  A node with more than SURV survivors is
// queued for the block merge (merge_kernel).  Same result as merging all
// candidates.  Persistent: each warp takes nodes grid-stride, so a block
// meets its barrier once at the end instead of waiting for its slowest node.
// SURV is 512, or 1024 while the previous merge queued more than n/32 nodes
// (the first iterations, when the pools are filling): twice the shared memory
// per warp and fewer warps per SM, but fewer nodes left to the block merge;
// refinement merges, with few survivors per node, take 128.
// With CREDIT (NN-descent merges) every survivor also keeps the index of its
// candidate slot (16 bits, CB <= 8192) and moves with its key through the
// sort; before the survivors are deduplicated, each distinct survivor placed
// at rank < K loads the joiners of its copies (beside their keys) and
// credits the lowest.  Three blocks of eight warps still share an SM; with
// 1024 survivor slots a block has seven warps so that two blocks share one.
constexpr int MW_WARPS = 8;
__host__ __device__ constexpr int merge_warps(int surv, bool credit) { return surv == 1024 && credit ? 7 : MW_WARPS; }
__host__ __device__ constexpr size_t merge_warp_bytes(uint32_t cap, int surv, bool credit) {
    return ((size_t)cap * 8 + (size_t)surv * 8 + 16 + (credit ? (size_t)surv * 2 : 0) + 15) & ~(size_t)15;
}

template <int SURV, bool CREDIT>
__global__ void __launch_bounds__(MW_WARPS * 32) merge_warp_kernel(MergeArgs a, uint32_t N, uint32_t *big_list,
                                                                  uint32_t *big_cnt) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    const size_t per_warp = merge_warp_bytes(a.cap, SURV, CREDIT);
    unsigned char *base = smem + w * per_warp;
    uint64_t *s_pool = reinterpret_cast<uint64_t *>(base);
    uint64_t *s_sv = s_pool + a.cap;         // survivors (keys without flags)
    uint64_t *s_last = s_sv + SURV;          // key landing at rank limit-1
    uint16_t *s_j = reinterpret_cast<uint16_t *>(s_last + 2); // CREDIT: each survivor's candidate slot
    __shared__ unsigned long long s_stat[4]; // flagged, inserted, candidates, entries
    if (threadIdx.x < 4) s_stat[threadIdx.x] = 0;
    __syncthreads();
    constexpr int NW = merge_warps(SURV, CREDIT);
    for (uint32_t node = blockIdx.x * NW + w; node < N; node += gridDim.x * NW) {
        const uint32_t raw = a.cand_cnt[node];
        // a refinement round leaves most pools without candidates: their pool,
        // count and radius stand (an NN-descent merge still counts every
        // pool's flagged entries for its delta, so it visits them all)
        if (!CREDIT && raw == 0) continue;
        const uint32_t nc = min(raw, a.CB);
        const uint32_t np = min(a.pool_cnt[node], a.limit);
        uint64_t *gp = a.pool + (uint64_t)node * a.cap;
        const uint64_t *gc = a.cand + 2 * (uint64_t)node * a.CB; // keys at even words
#pragma unroll 4
        for (uint32_t i = lane; i < np; i += 32) s_pool[i] = gp[i];
        // candidates in groups of 128 (four per lane), the next group's loads in
        // flight while this group is searched
        constexpr int CG = 4;
        uint64_t nxt[CG];
#pragma unroll
        for (int u = 0; u < CG; ++u) {
            const uint32_t j = 32 * u + lane;
            nxt[u] = j < nc ? gc[2 * j] : KCNA_EMPTY_KEY;
        }
        __syncwarp();
        // survivors: not in the pool, landing below limit
        uint32_t ns = 0;
        for (uint32_t b0 = 0; b0 < nc; b0 += 32 * CG) {
            uint64_t cur[CG];
#pragma unroll
            for (int u = 0; u < CG; ++u) {
                cur[u] = nxt[u];
                const uint32_t j = b0 + 32 * CG + 32 * u + lane;
                nxt[u] = j < nc ? gc[2 * j] : KCNA_EMPTY_KEY;
            }
#pragma unroll
            for (int u = 0; u < CG; ++u) {
                const uint32_t j = b0 + 32 * u + lane;
                bool surv = false;
                const uint64_t k = kcna_key_noflags(cur[u]);
                if (j < nc && k != KCNA_EMPTY_KEY_NOFLAGS) {
                    const int b = kcna_lower_bound(s_pool, (int)np, k);
                    surv = (uint32_t)b < a.limit && !(b < (int)np && (s_pool[b] >> 2) == (k >> 2));
                }
                const unsigned m = __ballot_sync(KCNA_FULL, surv);
                const uint32_t pos = ns + __popc(m & kcna_lanemask_lt());
                if (surv && pos < (uint32_t)SURV) {
                    s_sv[pos] = k;
                    if (CREDIT) s_j[pos] = (uint16_t)j;
                }
                ns += __popc(m);
            }
        }
        if (ns > (uint32_t)SURV) {
            if (lane == 0) big_list[atomicAdd(big_cnt, 1u)] = node;
        } else {
            uint32_t nu = 0; // distinct survivors
            if (ns > 0) {
                __syncwarp();
                if (CREDIT) {
                    kcna_warp_sort_n<true>(s_sv, s_j, (int)ns);
                    // copies of one key are adjacent: each distinct survivor whose
                    // rank (distinct index + position in the pool) is below K
                    // credits the lowest joiner among its copies.  Four batches of
                    // 32 at a time: their first joiners are loaded together, so the
                    // L2 round trips overlap.
                    uint32_t q0 = 0;
                    for (uint32_t b0 = 0; b0 < ns; b0 += 128) {
                        uint64_t kv[4];
                        uint32_t bv[4];
                        bool cr[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const uint32_t j = b0 + 32 * u + lane;
                            const uint64_t k = j < ns ? s_sv[j] : KCNA_EMPTY_KEY;
                            const uint64_t prev = j > 0 && j < ns ? s_sv[j - 1] : KCNA_EMPTY_KEY;
                            const bool start = j < ns && (j == 0 || (prev >> 2) != (k >> 2));
                            const unsigned m = __ballot_sync(KCNA_FULL, start);
                            const uint32_t q = q0 + __popc(m & kcna_lanemask_lt());
                            q0 += __popc(m);
                            cr[u] = start && q + (uint32_t)kcna_lower_bound(s_pool, (int)np, k) < a.K;
                            kv[u] = k;
                            bv[u] = cr[u] ? (uint32_t)gc[2 * s_j[j] + 1] : KCNA_NONE;
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            if (!cr[u]) continue;
                            uint32_t best = bv[u];
                            for (uint32_t x = b0 + 32 * u + lane + 1; x < ns && (s_sv[x] >> 2) == (kv[u] >> 2); ++x)
                                best = min(best, (uint32_t)gc[2 * s_j[x] + 1]);
                            if (best < a.n_nodes) a.found[best] = 1;
                        }
                    }
                    __syncwarp();
                } else {
                    kcna_warp_sort_n<false>(s_sv, nullptr, (int)ns);
                }
                // drop repeats among survivors (same distance and id are adjacent);
                // compaction moves entries down, so the previous key comes from
                // registers, not from the array being rewritten
                uint64_t carry = KCNA_EMPTY_KEY;
                for (uint32_t b0 = 0; b0 < ns; b0 += 32) {
                    const uint32_t j = b0 + lane;
                    const uint64_t k = j < ns ? s_sv[j] : KCNA_EMPTY_KEY;
                    uint64_t prev = __shfl_up_sync(KCNA_FULL, k, 1);
                    if (lane == 0) prev = carry;
                    const bool keep = j < ns && (j == 0 || (prev >> 2) != (k >> 2));
                    const unsigned m = __ballot_sync(KCNA_FULL, keep);
                    carry = __shfl_sync(KCNA_FULL, k, 31);
                    __syncwarp();
                    if (keep) s_sv[nu + __popc(m & kcna_lanemask_lt())] = k;
                    nu += __popc(m);
                    __syncwarp();
                }
            }
            const uint32_t newcnt = min(a.limit, np + nu);
            unsigned long long flagged = 0;
            if (lane == 0) *s_last = KCNA_EMPTY_KEY;
            __syncwarp();
            // pool entries: shifted by the survivors below them
            for (uint32_t i = lane; i < np; i += 32) {
                const uint64_t k = s_pool[i];
                const uint32_t sh = nu ? (uint32_t)kcna_lower_bound(s_sv, (int)nu, kcna_key_noflags(k)) : 0u;
                const uint32_t r = i + sh;
                if (r < newcnt) {
                    if (sh) gp[r] = k;
                    if (r < a.K && (k & KCNA_FLAG_NEW)) ++flagged;
                    if (r + 1 == a.limit) *s_last = k;
                }
            }
            // survivors at their rank
            unsigned long long placed = 0;
            for (uint32_t j = lane; j < nu; j += 32) {
                const uint64_t k = s_sv[j];
                const uint32_t r = j + (uint32_t)kcna_lower_bound(s_pool, (int)np, k);
                if (r < newcnt) {
                    gp[r] = k | KCNA_FLAG_NEW | KCNA_FLAG_ISNEW;
                    ++placed;
                    if (r < a.K) ++flagged;
                    if (r + 1 == a.limit) *s_last = k;
                }
            }
            flagged = kcna_warp_sum(flagged);
            placed = kcna_warp_sum(placed);
            __syncwarp();
            if (lane == 0) {
                if (flagged) atomicAdd(&s_stat[0], flagged);
                if (placed) atomicAdd(&s_stat[1], placed);
                atomicAdd(&s_stat[2], (unsigned long long)nc);
                atomicAdd(&s_stat[3], (unsigned long long)newcnt);
                if (raw > a.CB) atomicAdd(a.counters + 2, (unsigned long long)(raw - a.CB));
                a.pool_cnt[node] = newcnt;
                a.cand_cnt[node] = 0;
                a.radius[node] = newcnt >= a.limit ? kcna_key_dist(*s_last) : __uint_as_float(0x7F800000u);
            }
        }
        __syncwarp(); // the next node reuses this warp's shared memory
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_stat[0]) atomicAdd(a.counters + 1, s_stat[0]);
        if (s_stat[1]) atomicAdd(a.counters + 3, s_stat[1]);
        if (s_stat[2]) atomicAdd(a.counters + 7, s_stat[2]);
        if (s_stat[3]) atomicAdd(a.counters + 9, s_stat[3]);
    }
}

// In-place exclusive scan of data[0..n) by the whole block; data[n] receives
// the total.  s_warp holds blockDim.x/32 words.
__device__ uint32_t block_exclusive_scan(uint32_t *data, int n, uint32_t *s_warp) {
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per;
    uint32_t local = 0;
    for (int i = 0; i < per && b + i < n; ++i) local += data[b + i];
    uint32_t incl = local;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(KCNA_FULL, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            uint32_t t = s_warp[i];
            s_warp[i] = run;
            run += t;
        }
    }
    __syncthreads();
    uint32_t run = s_warp[w] + incl - local;
    for (int i = 0; i < per && b + i < n; ++i) {
        uint32_t t = data[b + i];
        data[b + i] = run;
        run += t;
    }
    if (threadIdx.x == blockDim.x - 1) data[n] = run;
    __syncthreads();
    return data[n];
}

// Block merge of nodes with many candidates (queued by merge_warp_kernel).
// Each candidate is placed by binary search into the gap of the sorted pool
// it falls in (its bucket: the number of pool entries below it); candidates
// equal to a pool entry or with bucket >= limit are dropped.  A counting sort
// by bucket then an insertion sort inside each bucket (block bitonic for the
// rare bucket above 32 entries) leave all candidates sorted, since buckets
// are ordered; duplicates are then adjacent.  Final position of pool entry i
// = i + kept candidates in buckets 0..i; of a kept candidate in bucket b =
// b + kept candidates before it.  Work is O(c log L + L) instead of a full
// sort of the candidates.
__global__ void __launch_bounds__(MT) merge_kernel(MergeArgs a, const uint32_t *big_list, const uint32_t *big_cnt) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int cbp = kcna_pow2_ceil_d((int)a.CB);
    uint64_t *s_pool = reinterpret_cast<uint64_t *>(smem); // cap
    uint64_t *s_c = s_pool + a.cap;                        // cbp (candidate keys, then bitonic scratch)
    uint64_t *s_sorted = s_c + cbp;                        // cbp
    uint32_t *s_b = reinterpret_cast<uint32_t *>(s_sorted + cbp); // cbp  bucket per candidate, then scratch
    uint32_t *s_ss = s_b + cbp;                            // cbp  joiner of each sorted candidate (credit)
    uint32_t *s_hist = s_ss + cbp;                         // cap + 2
    uint32_t *s_off = s_hist + a.cap + 2;                  // cap + 2
    uint32_t *s_giant = s_off + a.cap + 2;                 // cap + 2
    uint32_t *s_kept = reinterpret_cast<uint32_t *>(s_c);  // cbp + 1, once s_c's sorting is done
    const bool credit = a.credit != 0;
    __shared__ uint32_t s_warp[MT / 32];
    __shared__ uint32_t s_ngiant;
    __shared__ unsigned long long s_flagged;
    for (uint32_t bi = blockIdx.x; bi < *big_cnt; bi += gridDim.x) {
        __syncthreads();
        const uint32_t node = big_list[bi];
        const uint32_t raw = a.cand_cnt[node];
        const uint32_t nc = min(raw, a.CB);
        const uint32_t np = min(a.pool_cnt[node], a.limit);
        uint64_t *gp = a.pool + (uint64_t)node * a.cap;
        const uint64_t *gc = a.cand + 2 * (uint64_t)node * a.CB; // keys at even words
        if (threadIdx.x == 0) {
            s_flagged = 0;
            s_ngiant = 0;
        }
        for (uint32_t i = threadIdx.x; i < np; i += MT) s_pool[i] = gp[i];
        for (uint32_t i = threadIdx.x; i <= np + 1; i += MT) s_hist[i] = 0;
        __syncthreads();
        // bucket of every candidate
        for (uint32_t j = threadIdx.x; j < nc; j += MT) {
            const uint64_t k = kcna_key_noflags(gc[2 * j]);
            s_c[j] = k;
            const int b = kcna_lower_bound(s_pool, (int)np, k);
            const bool dup = b < (int)np && (s_pool[b] >> 2) == (k >> 2);
            if (dup || b >= (int)a.limit || k == KCNA_EMPTY_KEY_NOFLAGS) {
                s_b[j] = KCNA_NONE;
            } else {
                s_b[j] = (uint32_t)b;
                atomicAdd(&s_hist[b], 1u);
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i <= np; i += MT) s_off[i] = s_hist[i];
        __syncthreads();
        const uint32_t total = block_exclusive_scan(s_off, (int)np + 1, s_warp); // s_off[np+1] = total
        if (total == 0) { // nothing new: the pool stays as it is in memory
            unsigned long long f = 0;
            for (uint32_t i = threadIdx.x; i < np && i < a.K; i += MT) f += (s_pool[i] & KCNA_FLAG_NEW) ? 1 : 0;
            f = kcna_warp_sum(f);
            if ((threadIdx.x & 31) == 0 && f) atomicAdd(&s_flagged, f);
            __syncthreads();
            if (threadIdx.x == 0) {
                atomicAdd(a.counters + 1, s_flagged);
                if (raw > a.CB) atomicAdd(a.counters + 2, (unsigned long long)(raw - a.CB));
                atomicAdd(a.counters + 7, (unsigned long long)nc);
                atomicAdd(a.counters + 9, (unsigned long long)np);
                a.pool_cnt[node] = np;
                a.cand_cnt[node] = 0;
                a.radius[node] = np >= a.limit ? kcna_key_dist(s_pool[a.limit - 1]) : __uint_as_float(0x7F800000u);
            }
            continue;
        }
        for (uint32_t i = threadIdx.x; i <= np; i += MT) s_hist[i] = 0;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < nc; j += MT) {
            const uint32_t b = s_b[j];
            if (b != KCNA_NONE) {
                const uint32_t q = s_off[b] + atomicAdd(&s_hist[b], 1u);
                s_sorted[q] = s_c[j];
                s_ss[q] = credit ? (uint32_t)gc[2 * j + 1] : 0u;
            }
        }
        __syncthreads();
        // sort inside buckets, by key then joiner
        for (uint32_t b = threadIdx.x; b <= np; b += MT) {
            const uint32_t lo = s_off[b], hi = s_off[b + 1];
            if (hi - lo > 32) {
                s_giant[atomicAdd(&s_ngiant, 1u)] = b;
            } else {
                for (uint32_t x = lo + 1; x < hi; ++x) {
                    const uint64_t v = s_sorted[x];
                    const uint32_t vs = s_ss[x];
                    uint32_t y = x;
                    while (y > lo && (s_sorted[y - 1] > v || (s_sorted[y - 1] == v && s_ss[y - 1] > vs))) {
                        s_sorted[y] = s_sorted[y - 1];
                        s_ss[y] = s_ss[y - 1];
                        --y;
                    }
                    s_sorted[y] = v;
                    s_ss[y] = vs;
                }
            }
        }
        __syncthreads();
        const uint32_t ng = s_ngiant;
        for (uint32_t g = 0; g < ng; ++g) {
            const uint32_t b = s_giant[g];
            const uint32_t lo = s_off[b], len = s_off[b + 1] - lo;
            const int p2 = kcna_pow2_ceil_d((int)len);
            for (int i = threadIdx.x; i < p2; i += MT) {
                s_c[i] = i < (int)len ? s_sorted[lo + i] : KCNA_EMPTY_KEY;
                s_b[i] = i < (int)len ? s_ss[lo + i] : KCNA_NONE; // s_b is free after the scatter
            }
            kcna_cta_bitonic_kv(s_c, s_b, p2);
            for (uint32_t i = threadIdx.x; i < len; i += MT) {
                s_sorted[lo + i] = s_c[i];
                s_ss[lo + i] = s_b[i];
            }
            __syncthreads();
        }
        // duplicates among candidates are now adjacent
        for (uint32_t j = threadIdx.x; j < total; j += MT)
            s_kept[j] = (j == 0 || (s_sorted[j - 1] >> 2) != (s_sorted[j] >> 2)) ? 1u : 0u;
        __syncthreads();
        const uint32_t kept = block_exclusive_scan(s_kept, (int)total, s_warp);
        const uint32_t newcnt = min(a.limit, np + kept);
        unsigned long long flagged = 0, placed = 0;
        for (uint32_t i = threadIdx.x; i < np; i += MT) {
            const uint64_t k = s_pool[i];
            const uint32_t r = i + s_kept[s_off[i + 1]];
            if (r < newcnt) {
                gp[r] = k;
                if (r < a.K && (k & KCNA_FLAG_NEW)) ++flagged;
            }
        }
        for (uint32_t j = threadIdx.x; j < total; j += MT) {
            if (s_kept[j + 1] == s_kept[j]) continue; // duplicate
            // bucket of sorted position j: last b with s_off[b] <= j
            int lo = 0, hi = (int)np + 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= j)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const uint32_t r = (uint32_t)lo + s_kept[j];
            if (r < newcnt) {
                gp[r] = s_sorted[j] | KCNA_FLAG_NEW | KCNA_FLAG_ISNEW;
                ++placed;
                if (r < a.K) {
                    ++flagged;
                    if (credit && s_ss[j] < a.n_nodes) a.found[s_ss[j]] = 1; // lowest joiner of this key
                }
            }
        }
        flagged = kcna_warp_sum(flagged);
        placed = kcna_warp_sum(placed);
        if ((threadIdx.x & 31) == 0 && flagged) atomicAdd(&s_flagged, flagged);
        if ((threadIdx.x & 31) == 0 && placed) atomicAdd(a.counters + 3, placed);
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(a.counters + 1, s_flagged);
            if (raw > a.CB) atomicAdd(a.counters + 2, (unsigned long long)(raw - a.CB));
            atomicAdd(a.counters + 7, (unsigned long long)nc);
            atomicAdd(a.counters + 9, (unsigned long long)newcnt);
            a.pool_cnt[node] = newcnt;
            a.cand_cnt[node] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0)
            a.radius[node] = newcnt >= a.limit ? kcna_key_dist(gp[a.limit - 1]) : __uint_as_float(0x7F800000u);
    }
}

// ---------------------------------------------------------------------------
// sample (update, src/kgraph.cpp:1118-1202)
// ---------------------------------------------------------------------------
__global__ void sample_m_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                uint32_t N, uint32_t S, const uint8_t *__restrict__ found, uint32_t *__restrict__ Mv,
                                float *__restrict__ radiusM) {
    const uint32_t n = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = kcna_lane();
    if (n >= N) return;
    const uint64_t *pr = pool + (uint64_t)n * cap;
    uint32_t L = pool_cnt[n];
    uint32_t M = Mv[n];
    if (found[n]) {
        uint32_t maxl = min(M + S, L);
        uint32_t c = 0, l = maxl; // l: smallest prefix holding S flagged entries, else maxl
        for (uint32_t b = 0; b < maxl; b += 32) {
            uint32_t i = b + lane;
            bool f = i < maxl && (pr[i] & KCNA_FLAG_NEW);
            unsigned mk = __ballot_sync(KCNA_FULL, f);
            uint32_t tot = __popc(mk);
            if (c + tot >= S) {
                // position of the S-th flagged entry in this chunk
                uint32_t needed = S - c;
                unsigned mm = mk;
                for (uint32_t t = 1; t < needed; ++t) mm &= mm - 1;
                l = b + __ffs(mm);
                break;
            }
            c += tot;
        }
        M = l;
    }
    if (M == 0) M = min(1u, L); // the reference aborts here (BOOST_VERIFY, :1148)
    if (lane == 0) {
        Mv[n] = M;
        radiusM[n] = M > 0 ? kcna_key_dist(pr[M - 1]) : 0.f;
    }
}

__global__ void sample_lists_kernel(uint64_t *__restrict__ pool, uint32_t cap, uint32_t N,
                                    const uint32_t *__restrict__ Mv, const float *__restrict__ radiusM,
                                    uint32_t *__restrict__ fwd_new, uint32_t fwd_new_cap,
                                    uint32_t *__restrict__ fwd_new_cnt, uint32_t *__restrict__ fwd_old,
                                    uint32_t fwd_old_cap, uint32_t *__restrict__ fwd_old_cnt,
                                    uint32_t *__restrict__ rnew, uint32_t *__restrict__ rnew_cnt,
                                    uint32_t *__restrict__ rold, uint32_t *__restrict__ rold_cnt, uint32_t RB,
                                    unsigned long long *counters) {
    const uint32_t n = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = kcna_lane();
    if (n >= N) return;
    uint64_t *pr = pool + (uint64_t)n * cap;
    const uint32_t M = Mv[n];
    uint32_t cn = 0, co = 0;
    for (uint32_t b = 0; b < M; b += 32) {
        uint32_t l = b + lane;
        uint64_t k = l < M ? pr[l] : 0;
        bool valid = l < M;
        bool isnew = valid && (k & KCNA_FLAG_NEW);
        bool isold = valid && !(k & KCNA_FLAG_NEW);
        uint32_t id = kcna_key_id(k);
        float dd = kcna_key_dist(k);
        unsigned mn = __ballot_sync(KCNA_FULL, isnew), mo = __ballot_sync(KCNA_FULL, isold);
        if (isnew) {
            uint32_t p = cn + __popc(mn & kcna_lanemask_lt());
            if (p < fwd_new_cap) {
                fwd_new[(uint64_t)n * fwd_new_cap + p] = id;
                pr[l] = k & ~KCNA_FLAG_NEW; // used in a join from now on
            }
        }
        if (isold) {
            uint32_t p = co + __popc(mo & kcna_lanemask_lt());
            if (p < fwd_old_cap) fwd_old[(uint64_t)n * fwd_old_cap + p] = id;
        }
        // reverse edge n -> id only when n lies outside id's own join prefix
        if (valid && id < N && dd > radiusM[id]) {
            if (isnew) {
                uint32_t p = atomicAdd(rnew_cnt + id, 1u);
                if (p < RB)
                    rnew[(uint64_t)id * RB + p] = n;
                else
                    atomicAdd(counters + 12, 1ull); // dropped: which ones depends on timing
            } else {
                uint32_t p = atomicAdd(rold_cnt + id, 1u);
                if (p < RB)
                    rold[(uint64_t)id * RB + p] = n;
                else
                    atomicAdd(counters + 12, 1ull);
            }
        }
        cn += __popc(mn);
        co += __popc(mo);
    }
    if (lane == 0) {
        if (cn > fwd_new_cap) atomicAdd(counters + 4, (unsigned long long)(cn - fwd_new_cap));
        fwd_new_cnt[n] = min(cn, fwd_new_cap);
        fwd_old_cnt[n] = min(co, fwd_old_cap);
    }
}

// Random subset of R reverse entries (the reference shuffles rnn_* and keeps
// R, src/kgraph.cpp:1183-1201): each entry gets the priority
// hash(seed, iteration, node, id) and the R smallest priorities stay, in
// priority order.  The subset depends only on the set of entries, not on the
// order in which sample_lists_kernel's atomics appended them, so a run is
// reproducible as long as no list overflows RB.  Warp per list; lists of at
// most R entries are left as they are.
constexpr int SEL_WARPS = 8;
__global__ void __launch_bounds__(SEL_WARPS * 32) select_reverse_kernel(uint32_t *__restrict__ rnew,
                                                                       uint32_t *__restrict__ rnew_cnt,
                                                                       uint32_t *__restrict__ rold,
                                                                       uint32_t *__restrict__ rold_cnt, uint32_t N,
                                                                       uint32_t RB, uint32_t R, uint64_t seed,
                                                                       uint32_t iter, int P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t *s = reinterpret_cast<uint64_t *>(smem) + (size_t)w * P;
    const uint64_t item = (uint64_t)blockIdx.x * SEL_WARPS + w; // list index: node * 2 + old
    if (item >= 2ull * N) return;
    const uint32_t node = (uint32_t)(item >> 1), old = (uint32_t)(item & 1);
    uint32_t *list = (old ? rold : rnew) + (uint64_t)node * RB;
    uint32_t *cnt = (old ? rold_cnt : rnew_cnt) + node;
    const uint32_t m = min(*cnt, RB);
    if (m <= R) {
        if (lane == 0) *cnt = m; // never more than the stored entries
        return;
    }
    const uint64_t stream = join_reverse_stream(iter, node, old);
    for (int i = lane; i < P; i += 32) {
        if (i < (int)m) {
            const uint32_t id = list[i];
            s[i] = ((uint64_t)kcna_rand32(seed, stream, id) << 32) | id;
        } else {
            s[i] = KCNA_EMPTY_KEY;
        }
    }
    kcna_warp_bitonic(s, P);
    for (uint32_t i = lane; i < R; i += 32) list[i] = (uint32_t)(s[i] & 0xFFFFFFFFull);
    if (lane == 0) *cnt = R;
}

// BF16 screen mode: every candidate the screening join emitted is recomputed
// with the canonical FP32 chain from the FP32 rows, unless its id is already
// in the target's pool: such a repeat carries the pool entry's own distance
// (the chain is symmetric), so the merge would drop it as equal to that entry,
// and it becomes an empty key without a recompute.  A recomputed candidate
// beyond the target's radius becomes an empty key too (the merges skip those).
// Warp per target: the target's row in shared memory and its first np pool
// ids (np = min(count, limit), the entries the merge compares against) in an
// open-addressing table of ht slots; lane per candidate.  ht = 0 skips the
// repeat test.  (Adding the candidate ids to the table as well, to skip
// repeats within the buffer, was measured slower: the larger table costs
// occupancy and the inserts cost atomics.)
__global__ void __launch_bounds__(256) rescore_kernel(const float *__restrict__ X, int ld, uint32_t N,
                                                      uint64_t *__restrict__ cand, const uint32_t *__restrict__ cand_cnt,
                                                      uint32_t CB, const float *__restrict__ radius,
                                                      const uint64_t *__restrict__ pool,
                                                      const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                                      uint32_t limit, uint32_t ht, unsigned long long *rescored,
                                                      unsigned long long *repeats) {
    extern __shared__ __align__(16) float s_rows[]; // 8 warps x ld, then 8 warps x ht table slots
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t t = blockIdx.x * 8 + w;
    if (t >= N) return;
    float *xt = s_rows + (size_t)w * ld;
    uint32_t *tab = reinterpret_cast<uint32_t *>(s_rows + (size_t)8 * ld) + (size_t)w * ht;
    for (int k = lane; k < ld; k += 32) xt[k] = X[(uint64_t)t * ld + k];
    if (ht) {
        for (uint32_t h = lane; h < ht; h += 32) tab[h] = KCNA_NONE;
        __syncwarp();
        const uint32_t np = min(pool_cnt[t], min(limit, cap));
        for (uint32_t i = lane; i < np; i += 32) {
            const uint32_t id = kcna_key_id(pool[(uint64_t)t * cap + i]);
            uint32_t h = (id * 0x9E3779B1u) & (ht - 1);
            for (uint32_t probe = 0; probe < ht; ++probe, h = (h + 1) & (ht - 1)) {
                const uint32_t old = atomicCAS(&tab[h], KCNA_NONE, id);
                if (old == KCNA_NONE || old == id) break;
            }
        }
    }
    __syncwarp();
    const uint32_t nc = min(cand_cnt[t], CB);
    const float rad = radius[t];
    uint64_t *buf = cand + 2 * (uint64_t)t * CB; // keys at even words
    const float4 *x4 = reinterpret_cast<const float4 *>(xt);
    unsigned long long n = 0, rep = 0;
    for (uint32_t j = lane; j < nc; j += 32) {
        const uint64_t k = buf[2 * j];
        if (kcna_key_noflags(k) == KCNA_EMPTY_KEY_NOFLAGS) continue;
        const uint32_t id = kcna_key_id(k);
        bool in_pool = false;
        if (ht) {
            uint32_t h = (id * 0x9E3779B1u) & (ht - 1);
            for (uint32_t probe = 0; probe < ht; ++probe, h = (h + 1) & (ht - 1)) {
                const uint32_t e = tab[h];
                if (e == id) in_pool = true;
                if (e == id || e == KCNA_NONE) break;
            }
        }
        if (in_pool) {
            buf[2 * j] = KCNA_EMPTY_KEY;
            ++rep;
            continue;
        }
        const float4 *xc = reinterpret_cast<const float4 *>(X + (uint64_t)id * ld);
        float d = 0.f;
        for (int q = 0; q < (ld >> 2); ++q) d = kcna_acc4(d, x4[q], __ldg(xc + q));
        buf[2 * j] = d <= rad ? kcna_key(d, id, kcna_key_flags(k)) : KCNA_EMPTY_KEY;
        ++n;
    }
    n = kcna_warp_sum(n);
    rep = kcna_warp_sum(rep);
    if (lane == 0 && n) atomicAdd(rescored, n);
    if (lane == 0 && rep) atomicAdd(repeats, rep);
}

// control recall: |pool[0..min(cnt,K)) ∩ exact[0..K)| per control
__global__ void control_recall_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                      uint32_t cap, const uint32_t *__restrict__ controls,
                                      const uint32_t *__restrict__ knn, uint32_t knn_k, uint32_t K,
                                      unsigned long long *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *s = reinterpret_cast<uint64_t *>(smem);
    const uint32_t c = blockIdx.x, id = controls[c];
    const int p = kcna_pow2_ceil_d((int)K);
    for (int i = threadIdx.x; i < p; i += blockDim.x) s[i] = i < (int)K ? knn[(uint64_t)c * knn_k + i] : KCNA_EMPTY_KEY;
    kcna_cta_bitonic(s, p);
    uint32_t lim = min(pool_cnt[id], K);
    unsigned long long f = 0;
    for (uint32_t i = threadIdx.x; i < lim; i += blockDim.x) {
        uint64_t q = kcna_key_id(pool[(uint64_t)id * cap + i]);
        int lb = kcna_lower_bound(s, (int)K, q);
        if (lb < (int)K && s[lb] == q) ++f;
    }
    f = kcna_warp_sum(f);
    if ((threadIdx.x & 31) == 0 && f) atomicAdd(out, f);
}

__global__ void set_radius_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                  uint32_t cap, uint32_t N, uint32_t limit, float *__restrict__ radius) {
    uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    radius[n] = pool_cnt[n] >= limit ? kcna_key_dist(pool[(uint64_t)n * cap + limit - 1]) : __uint_as_float(0x7F800000u);
}

size_t join_smem_bytes(uint32_t capA, uint32_t capB) {
    return (size_t)(128 * JKP + JCOLS * JKP + 128 * (JCOLS + 1)) * sizeof(float) + (size_t)capA * 4 * 2 +
           (size_t)capB * 4;
}
size_t merge_smem_bytes(uint32_t cap, uint32_t CB) {
    size_t cp = (size_t)kcna_pow2_ceil((int)CB);
    return cap * 8 + cp * 8 * 2 + cp * 4 * 2 + (size_t)(cap + 2) * 4 * 3;
}

} // namespace

kcna_status kcna_nnd_alloc(kcna_ctx *c, const kcna_params *p, uint32_t maxl) {
    const uint64_t N = c->n;
    c->cap = maxl;
    c->S = p->S;
    c->Rr = p->R;
    // reverse-list buffer: 2R entries (at most 4 per join thread, 1024)
    const char *rb = getenv("KCNA_REV_CAP");
    c->RB = std::min<uint32_t>(std::max<uint32_t>(rb ? (uint32_t)atoi(rb) : 2 * p->R, std::max<uint32_t>(p->R, 32)), 1024);
    c->RB = (c->RB + 3) & ~3u; // rows of 16-byte multiples (bulk copies in the Gram-tile join)
    const char *cb = getenv("KCNA_CAND_CAP");
    uint32_t CB = cb ? (uint32_t)atoi(cb) : 4 * std::max<uint32_t>(p->L, 64);
    CB = std::min<uint32_t>(std::max<uint32_t>(CB, 64), 8192);
    c->CB = (uint32_t)kcna_pow2_ceil((int)CB);
    c->fwd_new_cap = (std::max<uint32_t>(2 * p->S, 64) + 3) & ~3u;
    c->fwd_old_cap = (std::max<uint32_t>(p->L, 1) + 3) & ~3u;
    // two spare entries: the tile prunes copy pool prefixes from an even index
    // in 16-byte units, which can reach one entry past the last row
    KCNA_TRY(kcna_alloc(c, &c->pool, N * c->cap + 2, "pool"));
    KCNA_TRY(kcna_alloc(c, &c->pool_cnt, N, "pool_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->radius, N, "radius"));
    KCNA_TRY(kcna_alloc(c, &c->M, N, "M"));
    KCNA_TRY(kcna_alloc(c, &c->radiusM, N, "radiusM"));
    KCNA_TRY(kcna_alloc(c, &c->found, N, "found"));
    KCNA_TRY(kcna_alloc(c, &c->fwd_new, N * c->fwd_new_cap, "fwd_new"));
    KCNA_TRY(kcna_alloc(c, &c->fwd_new_cnt, N, "fwd_new_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->fwd_old, N * c->fwd_old_cap, "fwd_old"));
    KCNA_TRY(kcna_alloc(c, &c->fwd_old_cnt, N, "fwd_old_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->rnew, N * c->RB, "rnew"));
    KCNA_TRY(kcna_alloc(c, &c->rnew_cnt, N, "rnew_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->rold, N * c->RB, "rold"));
    KCNA_TRY(kcna_alloc(c, &c->rold_cnt, N, "rold_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->cand, 2 * N * c->CB, "candidate buffers"));
    KCNA_TRY(kcna_alloc(c, &c->cand_cnt, N, "cand_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->big_list, N, "merge queue"));
    KCNA_TRY(kcna_alloc(c, &c->big_cnt, 1, "merge queue count"));
    if (!c->counters) KCNA_TRY(kcna_alloc(c, &c->counters, 64, "counters"));
    cudaStream_t s = c->stream;
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->cand_cnt, 0, N * 4, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->rnew_cnt, 0, N * 4, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->rold_cnt, 0, N * 4, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->fwd_old_cnt, 0, N * 4, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->found, 0, N, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters, 0, 64 * 8, s), "memset"));
    return KCNA_OK;
}

kcna_status kcna_cand_alloc(kcna_ctx *c, const kcna_params *p) {
    if (c->cand && c->cand_cnt && c->big_list && c->big_cnt && c->counters) return KCNA_OK;
    const uint64_t N = c->n;
    const char *cb = getenv("KCNA_CAND_CAP");
    uint32_t CB = cb ? (uint32_t)atoi(cb) : 4 * std::max<uint32_t>(p->L, 64);
    CB = std::min<uint32_t>(std::max<uint32_t>(CB, 64), 8192);
    c->CB = (uint32_t)kcna_pow2_ceil((int)CB);
    KCNA_TRY(kcna_alloc(c, &c->cand, 2 * N * c->CB, "candidate buffers"));
    KCNA_TRY(kcna_alloc(c, &c->cand_cnt, N, "cand_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->big_list, N, "merge queue"));
    KCNA_TRY(kcna_alloc(c, &c->big_cnt, 1, "merge queue count"));
    if (!c->counters) KCNA_TRY(kcna_alloc(c, &c->counters, 64, "counters"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->cand_cnt, 0, N * 4, c->stream), "memset"));
    return KCNA_OK;
}

kcna_status kcna_nnd_init(kcna_ctx *c, const kcna_params *p) {
    if (p->S == 0 || p->S > 31) return kcna_fail(c, KCNA_E_ARG, "S must be in [1, 31]");
    KCNA_TRY(kcna_phase_begin(c));
    init_kernel<<<kcna_div_up(c->n, 4), 128, 0, c->stream>>>(c->X, (int)c->ld, c->n, p->S, c->cap, p->seed, c->pool,
                                                           c->pool_cnt, c->fwd_new, c->fwd_new_cap, c->fwd_new_cnt);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "init_kernel"));
    KCNA_TRY(kcna_pools_set_radius(c, p->L));
    // M = S (src/kgraph.cpp:1030)
    std::vector<uint32_t> Ms(c->n, p->S);
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->M, Ms.data(), (size_t)c->n * 4, cudaMemcpyHostToDevice, c->stream),
                             "M init"));
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_INIT));
    c->has_pools = true;
    return KCNA_OK;
}

kcna_status kcna_nnd_join(kcna_ctx *c, const kcna_params *p, int iter, uint64_t *n_comps) {
    JoinArgs a;
    a.X = c->X;
    a.ld = (int)c->ld;
    a.N = c->n;
    a.iter = (uint32_t)iter;
    a.seed = p->seed;
    a.R = p->R;
    a.RB = c->RB;
    a.fwd_new = c->fwd_new;
    a.fwd_new_cnt = c->fwd_new_cnt;
    a.fwd_new_cap = c->fwd_new_cap;
    a.fwd_old = c->fwd_old;
    a.fwd_old_cnt = c->fwd_old_cnt;
    a.fwd_old_cap = c->fwd_old_cap;
    a.rnew = c->rnew;
    a.rnew_cnt = c->rnew_cnt;
    a.rold = c->rold;
    a.rold_cnt = c->rold_cnt;
    a.radius = c->radius;
    a.cand = c->cand;
    a.cand_cnt = c->cand_cnt;
    a.CB = c->CB;
    a.found = c->found;
    a.counters = c->counters;
    a.capA = c->fwd_new_cap + std::min(p->R, c->RB);
    a.capB = c->fwd_old_cap + std::min(p->R, c->RB);
    a.err = c->d_err;
    size_t sm = join_smem_bytes(a.capA, a.capB);
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_kernel<RowsF32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "join smem attr"));
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(join_kernel<RowsB16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "join smem attr"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters, 0, 8 * 8, c->stream), "memset"));
    // found (src/kgraph.cpp:1104,1116): cleared for every node, then set by the
    // merge for the joiners whose candidates it inserts below K
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->found, 0, c->n, c->stream), "memset"));
    KCNA_TRY(kcna_phase_begin(c));
    if ((c->gram_exact || c->bf16_screen) && kcna_join_tc_fits(a)) {
        KCNA_TRY(kcna_join_tc_launch(c, a));
        if (c->bf16_screen) {
            const uint32_t limit = std::min(p->L, c->cap);
            uint32_t ht = 64; // the pool ids at half load at most
            while (ht < 2 * limit) ht <<= 1;
            size_t rs = (size_t)8 * c->ld * 4 + (size_t)8 * ht * 4;
            if (rs > 160 * 1024) { // very long pools: recompute every candidate
                ht = 0;
                rs = (size_t)8 * c->ld * 4;
            }
            KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(rescore_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                             (int)std::max<size_t>(rs, 48 * 1024)),
                                     "rescore smem attr"));
            rescore_kernel<<<kcna_div_up(c->n, 8), 256, rs, c->stream>>>(
                c->X, (int)c->ld, c->n, c->cand, c->cand_cnt, c->CB, c->radius, c->pool, c->pool_cnt, c->cap, limit,
                ht, c->counters + 13, c->counters + 14);
            KCNA_LAUNCHED(c);
            KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "rescore_kernel"));
        }
    } else {
        if (c->bf16_exact)
            join_kernel<<<c->n, JT, sm, c->stream>>>(a, RowsB16{c->Xh, (int)c->ld});
        else
            join_kernel<<<c->n, JT, sm, c->stream>>>(a, RowsF32{c->X, (int)c->ld});
        KCNA_LAUNCHED(c);
        KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "join_kernel"));
    }
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_JOIN));
    unsigned long long h[8] = {};
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(h, c->counters, 8 * 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "join sync"));
    if (n_comps) *n_comps = h[0];
    c->join_rows += h[5];
    c->cand_emitted += h[6];
    return KCNA_OK;
}

kcna_status kcna_merge(kcna_ctx *c, uint32_t limit, uint32_t K, uint64_t *overflow, uint64_t *flagged_topk,
                       uint64_t *merged, uint64_t *inserted, bool credit_found) {
    MergeArgs a;
    a.pool = c->pool;
    a.pool_cnt = c->pool_cnt;
    a.cap = c->cap;
    a.limit = std::min(limit, c->cap);
    a.K = K;
    a.radius = c->radius;
    a.cand = c->cand;
    a.cand_cnt = c->cand_cnt;
    a.CB = c->CB;
    a.counters = c->counters;
    a.credit = credit_found ? 1u : 0u;
    a.found = c->found;
    a.n_nodes = c->n;
    size_t sm = merge_smem_bytes(c->cap, c->CB);
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "merge smem attr"));
    const char *wd = getenv("KCNA_MERGE_WIDE_DIV"); // tuning override of the threshold below
    const uint32_t wide_div = wd ? std::max(1, atoi(wd)) : 32; // 64 and 16 measured slower at C2 1M
    const bool wide = c->merge_big_last > c->n / wide_div; // many nodes overflowed the survivor buffer last time
    const char *sv = getenv("KCNA_MERGE_SURV");   // tuning override: 128, 512 or 1024
    // refinement merges (no credit) meet few survivors per node: 128 slots per
    // warp, so that five blocks instead of three share an SM
    const int surv = sv ? (atoi(sv) >= 1024 ? 1024 : atoi(sv) >= 512 ? 512 : 128)
                        : wide ? 1024 : credit_found ? 512 : 128;
    const int nw = merge_warps(surv, credit_found);
    const size_t smw = merge_warp_bytes(c->cap, surv, credit_found) * nw;
    auto launch_warp = [&](auto kern) -> kcna_status {
        KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)std::max<size_t>(smw, 48 * 1024)),
                                 "merge smem attr"));
        int mw_per_sm = 0;
        KCNA_TRY(kcna_cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mw_per_sm, kern, nw * 32, smw),
                                 "merge occupancy"));
        const uint32_t mw_grid = (uint32_t)std::min<uint64_t>(
            kcna_div_up(c->n, nw), (uint64_t)std::max(c->num_sms, 1) * std::max(mw_per_sm, 1));
        KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters, 0, 10 * 8, c->stream), "memset"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->big_cnt, 0, 4, c->stream), "memset"));
        KCNA_TRY(kcna_phase_begin(c));
        kern<<<mw_grid, nw * 32, smw, c->stream>>>(a, c->n, c->big_list, c->big_cnt);
        return KCNA_OK;
    };
    // the template must match the shared memory sized above
    if (credit_found)
        KCNA_TRY(surv == 1024 ? launch_warp(merge_warp_kernel<1024, true>) : launch_warp(merge_warp_kernel<512, true>));
    else
        KCNA_TRY(surv == 1024  ? launch_warp(merge_warp_kernel<1024, false>)
                 : surv == 512 ? launch_warp(merge_warp_kernel<512, false>)
                               : launch_warp(merge_warp_kernel<128, false>));
    merge_kernel<<<std::max(1, c->num_sms) * 4, MT, sm, c->stream>>>(a, c->big_list, c->big_cnt);
    c->launches += 2;
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "merge_kernel"));
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_MERGE));
    unsigned long long h[10] = {};
    uint32_t hb = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(h, c->counters, 10 * 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&hb, c->big_cnt, 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "merge sync"));
    c->merge_big_last = hb;
    c->cand_merged += h[7];
    c->pool_entries_merged += h[9];
    if (merged) *merged = h[7];
    if (inserted) *inserted = h[3];
    if (overflow) *overflow = h[2];
    if (flagged_topk) *flagged_topk = h[1];
    return KCNA_OK;
}

kcna_status kcna_nnd_sample(kcna_ctx *c, const kcna_params *p, int iter) {
    cudaStream_t s = c->stream;
    KCNA_TRY(kcna_phase_begin(c));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->rnew_cnt, 0, (size_t)c->n * 4, s), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->rold_cnt, 0, (size_t)c->n * 4, s), "memset"));
    sample_m_kernel<<<kcna_div_up(c->n, 8), 256, 0, s>>>(c->pool, c->pool_cnt, c->cap, c->n, p->S, c->found, c->M,
                                                          c->radiusM);
    KCNA_LAUNCHED(c);
    sample_lists_kernel<<<kcna_div_up(c->n, 8), 256, 0, s>>>(c->pool, c->cap, c->n, c->M, c->radiusM, c->fwd_new,
                                                              c->fwd_new_cap, c->fwd_new_cnt, c->fwd_old,
                                                              c->fwd_old_cap, c->fwd_old_cnt, c->rnew, c->rnew_cnt,
                                                              c->rold, c->rold_cnt, c->RB, c->counters);
    KCNA_LAUNCHED(c);
    const int P = kcna_pow2_ceil((int)c->RB);
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(select_reverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     SEL_WARPS * P * 8),
                             "select smem attr"));
    select_reverse_kernel<<<kcna_div_up(2ull * c->n, SEL_WARPS), SEL_WARPS * 32, (size_t)SEL_WARPS * P * 8, s>>>(
        c->rnew, c->rnew_cnt, c->rold, c->rold_cnt, c->n, c->RB, p->R, p->seed, (uint32_t)iter, P);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "sample kernels"));
    return kcna_phase_end(c, KCNA_PHASE_SAMPLE);
}

kcna_status kcna_pools_set_radius(kcna_ctx *c, uint32_t limit) {
    set_radius_kernel<<<kcna_div_up(c->n, 256), 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, c->n,
                                                                      std::min(limit, c->cap), c->radius);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "set_radius");
}

// Controls: C random nodes and their exact MAXL-NN (GenerateControl,
// src/kgraph.cpp:363-387).  The nodes are the reference's own: the first C of
// 0..n-1 after std::random_shuffle driven by the C library's rand() in its
// initial state (the reference never seeds it), i.e. for i = 1..n-1 swap
// index[i] with index[rand() % (i + 1)].  The same generator runs here on a
// private state (random_r seeded with 1, the state rand() starts from), so
// the caller's rand() sequence is left alone; the order is cached per (n, C).
kcna_status kcna_controls_setup(kcna_ctx *c, const kcna_params *p, uint32_t maxl) {
    uint32_t C = std::min<uint32_t>(p->controls, c->n - 1);
    c->control_ids.clear();
    if (C == 0) return KCNA_OK;
    if (c->control_cache_n != c->n || c->control_cache.size() != C) {
        std::vector<uint32_t> idx(c->n);
        for (uint32_t i = 0; i < c->n; ++i) idx[i] = i;
        struct random_data rd;
        char state[128];
        std::memset(&rd, 0, sizeof rd);
        std::memset(state, 0, sizeof state);
        if (initstate_r(1u, state, sizeof state, &rd) != 0) return kcna_fail(c, KCNA_E_CUDA, "initstate_r failed");
        for (uint32_t i = 1; i < c->n; ++i) {
            int32_t r = 0;
            random_r(&rd, &r);
            std::swap(idx[i], idx[(uint32_t)r % (i + 1)]);
        }
        c->control_cache.assign(idx.begin(), idx.begin() + C);
        c->control_cache_n = c->n;
    }
    c->control_ids = c->control_cache;
    c->control_k = maxl;
    KCNA_TRY(kcna_alloc(c, &c->d_controls, C, "controls"));
    KCNA_TRY(kcna_alloc(c, &c->d_control_knn, (size_t)C * maxl, "control knn"));
    float *dd = nullptr, *rows = nullptr;
    KCNA_TRY(kcna_alloc(c, &dd, (size_t)C * maxl, "control dists"));
    KCNA_TRY(kcna_alloc(c, &rows, (size_t)C * c->ld, "control rows"));
    kcna_status st = kcna_phase_begin(c);
    if (st == KCNA_OK)
        st = kcna_cuda_check(c, cudaMemcpyAsync(c->d_controls, c->control_ids.data(), C * 4, cudaMemcpyHostToDevice,
                                                c->stream), "h2d");
    if (st == KCNA_OK) st = kcna_gather_rows(c, c->d_controls, C, rows);
    if (st == KCNA_OK) st = kcna_knn_device(c, rows, C, c->d_controls, maxl, c->d_control_knn, dd);
    if (st == KCNA_OK) st = kcna_phase_end(c, KCNA_PHASE_CONTROLS);
    kcna_release(c, dd);
    kcna_release(c, rows);
    return st;
}

kcna_status kcna_control_recall(kcna_ctx *c, uint32_t K, float *recall) {
    uint32_t C = (uint32_t)c->control_ids.size();
    if (C == 0) {
        *recall = 0.f;
        return KCNA_OK;
    }
    K = std::min(K, c->control_k);
    KCNA_TRY(kcna_phase_begin(c));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters + 8, 0, 8, c->stream), "memset"));
    size_t sm = (size_t)kcna_pow2_ceil((int)K) * 8;
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(control_recall_kernel,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "attr"));
    control_recall_kernel<<<C, 256, sm, c->stream>>>(c->pool, c->pool_cnt, c->cap, c->d_controls, c->d_control_knn,
                                                     c->control_k, K, c->counters + 8);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "control_recall"));
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_CONTROLS));
    unsigned long long h = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&h, c->counters + 8, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "recall sync"));
    *recall = (float)((double)h / ((double)C * K));
    return KCNA_OK;
}

// The constructor loop of src/kgraph.cpp:1281-1459 with its stop rule
// (delta <= params.delta, recall >= params.recall, or I iterations).
kcna_status kcna_nndescent_run(kcna_ctx *c, const kcna_params *pin, kcna_stats *st) {
    kcna_params P = *pin;
    const uint32_t N = c->n;
    if (N < 3) return kcna_fail(c, KCNA_E_ARG, "need at least 3 rows");
    // parameter clamping, src/kgraph.cpp:1289-1327
    if (N <= P.controls) P.controls = N - 1;
    if (N <= P.L) P.L = N - 1;
    if (N <= P.S) P.S = N - 1;
    if (N <= P.search_L) P.search_L = N - 1;
    if (N <= P.search_K) P.search_K = N - 1;
    if (N <= P.K) {
        P.K = N - 1;
        P.loop_i = 0;
        P.S = N - 1;
        P.iterations = 0;
    }
    const uint32_t maxl = std::max(std::max(P.L, P.K), std::max(P.search_L, P.search_K));
    if (maxl > 1024) return kcna_fail(c, KCNA_E_ARG, "max(L, K, search_L, search_K) must be <= 1024");
    st->maxl = maxl;
    c->merge_big_last = c->n; // the first merges fill the pools: wide survivor buffers
    KCNA_TRY(kcna_nnd_alloc(c, &P, maxl));
    KCNA_TRY(kcna_controls_setup(c, &P, maxl));
    // join iterations count from 1 when the first lists come from an update step
    int iter_base = 0;
    if (P.learned_seed) {
        KCNA_TRY(kcna_seed_learned(c, &P, st));
        KCNA_TRY(kcna_seed_finish(c, &P));
        KCNA_TRY(kcna_control_recall(c, P.K, &st->seed_recall));
        kcna_log(c, &P, "learned seed: %.1f ms (training %.1f ms), loss %.3f -> %.3f, recall %.4f", st->seed_total_ms,
                 st->seed_train_ms, st->seed_loss_first, st->seed_loss_last, st->seed_recall);
        KCNA_TRY(kcna_nnd_sample(c, &P, 1));
        iter_base = 1;
    } else {
        KCNA_TRY(kcna_nnd_init(c, &P));
    }
    uint64_t comps_total = 0;
    st->stop_condition = 0;
    st->iterations = 0;
    for (uint32_t it = 0; it < P.iterations; ++it) {
        uint64_t comps = 0, overflow = 0, flagged = 0, merged = 0, inserted = 0;
        const double j0 = c->phase_ms[KCNA_PHASE_JOIN], m0 = c->phase_ms[KCNA_PHASE_MERGE];
        KCNA_TRY(kcna_nnd_join(c, &P, (int)it + iter_base, &comps));
        KCNA_TRY(kcna_merge(c, P.L, P.K, &overflow, &flagged, &merged, &inserted, true));
        if (it < KCNA_MAX_ITERS) {
            st->iter_join_ms[it] = c->phase_ms[KCNA_PHASE_JOIN] - j0;
            st->iter_merge_ms[it] = c->phase_ms[KCNA_PHASE_MERGE] - m0;
            st->iter_cand[it] = merged;
            st->iter_inserted[it] = inserted;
        }
        comps_total += comps;
        float delta = (float)((double)flagged / ((double)N * P.K));
        float recall = 0.f;
        KCNA_TRY(kcna_control_recall(c, P.K, &recall));
        if (it < KCNA_MAX_ITERS) {
            st->iter_recall[it] = recall;
            st->iter_delta[it] = delta;
            st->iter_time[it] = kcna_now() - c->t0;
            st->iter_cand_overflow[it] = overflow;
        }
        st->iterations = it + 1;
        kcna_log(c, &P, "iteration %u recall %.4f delta %.4f comps %llu overflow %llu t %.3f", it + 1, recall, delta,
                 (unsigned long long)comps, (unsigned long long)overflow, kcna_now() - c->t0);
        KCNA_TRY(kcna_check_device_err(c, "nndescent"));
        if (delta <= P.delta) {
            st->stop_condition = 1;
            break;
        }
        if (recall >= P.recall) {
            st->stop_condition = 2;
            break;
        }
        if (it + 1 >= P.iterations) break;
        KCNA_TRY(kcna_nnd_sample(c, &P, (int)it + 1 + iter_base));
    }
    st->n_comps = comps_total;
    // pairs screened on Gram tiles; in screen mode the candidates among them were recomputed in FP32
    st->screened_pairs = (c->gram_exact || c->bf16_screen) ? comps_total : 0;
    unsigned long long resc = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&resc, c->counters + 13, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    st->rescored_pairs = resc;
    unsigned long long rev_drop = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&rev_drop, c->counters + 12, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync"));
    st->rev_overflow = (uint32_t)std::min<unsigned long long>(rev_drop, 0xFFFFFFFFull);
    return KCNA_OK;
}
