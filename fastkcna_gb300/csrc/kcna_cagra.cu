// kcna_cagra.cu - CAGRA-style rank prune of the candidate pools into the graph.
//
// The reference's BuildCagra (src/kgraph.cpp:2818-2829; no build function
// calls it there) turns each node's K nearest pool entries into a graph of
// about K / 2 edges by counting detours instead of comparing distances:
//   route   (CagraComputeRoute, :2665-2757) route[j] = number of pairs (k, l)
//           with pool_i[k]'s own entry l equal to pool_i[j] and k, l < j;
//   keep    the prune_K = K / 2 entries with the fewest detours, equal counts
//           in rank order (sort_indexes, :62-76);
//   reverse (CagraReverse, :2759-2788) every kept edge i -> w gives w the entry
//           (i, rank of w in i's kept list), taken by increasing rank; equal
//           ranks by increasing source id (the reference sorts by rank alone,
//           leaving that order unspecified);
//   merge   (CagraMerge, :2790-2816) kept and reverse entries alternate until
//           prune_K are placed, one more when the last step places both;
//           a reverse entry carries d(i, source).
// With Ki = min(K, pool count), entries past a pool's count are absent.
//
// GPU form, four steps on the context's stream:
//   cagra_route_kernel  block per node: the node's first Ki pool ids in a
//                       shared-memory hash table (id -> rank), the K x K
//                       two-hop entries looked up in it (warp per one-hop
//                       node, lanes over its pool: coalesced 8-byte keys),
//                       detours counted with shared atomics, (route, rank)
//                       keys sorted, the kept ranks written and each kept
//                       target's in-degree counted;
//   exclusive scan of the in-degrees (kcna_graph.cu);
//   cagra_rev_fill_kernel  thread per kept edge: (rank << 32 | source) into
//                       the target's segment;
//   cagra_merge_kernel  block per node: the smallest reverse keys (the
//                       segment sorted in shared memory, or streamed through
//                       a 1024-key best set for hubs), then the interleaved
//                       row with every slot's position computed in closed form.
#include "kcna_internal.h"
#include "kcna_sort.cuh"

namespace {

constexpr int CG_THREADS = 256;
constexpr uint32_t CG_EMPTY = 0xFFFFFFFFu;
constexpr int CG_BEST = 1024; // merge: best-set size when a segment is streamed

__device__ __forceinline__ uint32_t cg_hash(uint32_t id) { return (id * 0x9E3779B1u) >> 7; }

// Kept ranks of node i (fwd[i * PK + r] = pool index) and the kept targets'
// in-degrees.  Shared: ids[K], table keys[HS], table ranks[HS], route[K],
// sort keys[P2] (P2 = K rounded up to a power of two, HS = 2 P2).
__global__ void __launch_bounds__(CG_THREADS) cagra_route_kernel(const uint64_t *__restrict__ pool,
                                                                 const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                                                 uint32_t N, uint32_t K, uint32_t PK, uint32_t P2,
                                                                 uint16_t *__restrict__ fwd, uint32_t *__restrict__ indeg,
                                                                 int *err) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *skey = reinterpret_cast<uint64_t *>(smem);       // P2
    uint32_t *ids = reinterpret_cast<uint32_t *>(skey + P2);   // K
    uint32_t *route = ids + K;                                  // K
    uint32_t *hkey = route + K;                                 // 2 P2
    uint32_t *hval = hkey + 2 * P2;                             // 2 P2
    const uint32_t i = blockIdx.x, HS = 2 * P2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = CG_THREADS / 32;
    if (i >= N) return;
    const uint32_t Ki = min(K, pool_cnt[i]);
    for (uint32_t h = tid; h < HS; h += CG_THREADS) hkey[h] = CG_EMPTY;
    __syncthreads();
    for (uint32_t j = tid; j < Ki; j += CG_THREADS) {
        const uint32_t id = kcna_key_id(pool[(uint64_t)i * cap + j]);
        ids[j] = id;
        route[j] = 0;
        uint32_t h = cg_hash(id) & (HS - 1);
        for (uint32_t probe = 0; probe < HS; ++probe, h = (h + 1) & (HS - 1))
            if (atomicCAS(&hkey[h], CG_EMPTY, id) == CG_EMPTY) {
                hval[h] = j;
                break;
            }
    }
    __syncthreads();
    // two-hop entries: pool_i[k]'s entry l, looked up among pool_i's ranks
    for (uint32_t k = warp; k < Ki; k += nw) {
        const uint32_t one = ids[k];
        if (one >= N) {
            kcna_set_err(err, KCNA_DERR_BOUNDS);
            continue;
        }
        const uint32_t Kl = min(K, pool_cnt[one]);
        const uint64_t *p1 = pool + (uint64_t)one * cap;
        for (uint32_t l = lane; l < Kl; l += 32) {
            const uint32_t two = kcna_key_id(__ldg(p1 + l));
            uint32_t h = cg_hash(two) & (HS - 1);
            for (uint32_t probe = 0; probe < HS; ++probe, h = (h + 1) & (HS - 1)) {
                const uint32_t key = hkey[h];
                if (key == CG_EMPTY) break;
                if (key == two) {
                    const uint32_t j = hval[h];
                    if (j > max(k, l)) atomicAdd(&route[j], 1u);
                    break;
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t j = tid; j < P2; j += CG_THREADS) skey[j] = j < Ki ? ((uint64_t)route[j] << 32) | j : ~0ull;
    kcna_cta_bitonic(skey, (int)P2);
    const uint32_t nk = min(PK, Ki);
    for (uint32_t r = tid; r < nk; r += CG_THREADS) {
        const uint32_t j = (uint32_t)(skey[r] & 0xFFFFFFFFull);
        fwd[(uint64_t)i * PK + r] = (uint16_t)j;
        const uint32_t w = ids[j];
        if (w < N)
            atomicAdd(indeg + w, 1u);
        else
            kcna_set_err(err, KCNA_DERR_BOUNDS);
    }
}

// Reverse entries: thread per kept edge (i, r) -> target's segment.
__global__ void cagra_rev_fill_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                      uint32_t cap, uint32_t N, uint32_t K, uint32_t PK,
                                      const uint16_t *__restrict__ fwd, const uint64_t *__restrict__ off,
                                      uint32_t *__restrict__ cursor, uint64_t *__restrict__ rev) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)N * PK) return;
    const uint32_t i = (uint32_t)(t / PK), r = (uint32_t)(t % PK);
    if (r >= min(PK, min(K, pool_cnt[i]))) return;
    const uint32_t w = kcna_key_id(pool[(uint64_t)i * cap + fwd[t]]);
    if (w >= N) return; // counted as an error by the route kernel
    const uint64_t pos = off[w] + atomicAdd(cursor + w, 1u);
    rev[pos] = ((uint64_t)r << 32) | i;
}

// Row of node i: kept entry t at t + min(t, m), reverse entry t at
// min(t + 1, nk) + t; a step t runs while the row holds fewer than PK
// entries, size_before(t) = min(t, nk) + min(t, m).
template <class R>
__global__ void __launch_bounds__(CG_THREADS) cagra_merge_kernel(R rows, const uint64_t *__restrict__ pool,
                                                                 const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                                                 uint32_t N, uint32_t K, uint32_t PK,
                                                                 const uint16_t *__restrict__ fwd,
                                                                 const uint64_t *__restrict__ off,
                                                                 const uint64_t *__restrict__ rev,
                                                                 uint32_t *__restrict__ g_ids, float *__restrict__ g_dist,
                                                                 uint32_t *__restrict__ g_deg, uint32_t W, int *err) {
    __shared__ uint64_t s[2 * CG_BEST];
    const uint32_t i = blockIdx.x;
    const int tid = threadIdx.x;
    if (i >= N) return;
    const uint32_t nk = min(PK, min(K, pool_cnt[i]));
    const uint64_t b = off[i];
    const uint32_t m = (uint32_t)(off[i + 1] - b);
    // reverse entries the row can take: steps run while fewer than PK are placed
    uint32_t T = 0;
    while ((T < nk || T < m) && min(T, nk) + min(T, m) < PK) ++T;
    const uint32_t need = min(T, m);
    // the `need` smallest (rank, source) keys in s[0 ..)
    if (m <= 2 * CG_BEST) {
        uint32_t p2 = 1;
        while (p2 < m) p2 <<= 1;
        for (uint32_t j = tid; j < p2; j += CG_THREADS) s[j] = j < m ? rev[b + j] : ~0ull;
        kcna_cta_bitonic(s, (int)p2);
    } else {
        for (uint32_t j = tid; j < CG_BEST; j += CG_THREADS) s[j] = ~0ull;
        for (uint32_t c0 = 0; c0 < m; c0 += CG_BEST) {
            __syncthreads();
            for (uint32_t j = tid; j < CG_BEST; j += CG_THREADS)
                s[CG_BEST + j] = c0 + j < m ? rev[b + c0 + j] : ~0ull;
            kcna_cta_bitonic(s, 2 * CG_BEST);
        }
    }
    const uint32_t deg = min(T, nk) + need;
    if (deg > W) {
        if (tid == 0) kcna_set_err(err, KCNA_DERR_DEGREE);
        return;
    }
    uint32_t *gi = g_ids + (uint64_t)i * W;
    float *gd = g_dist + (uint64_t)i * W;
    for (uint32_t t = tid; t < min(T, nk); t += CG_THREADS) {
        const uint64_t key = pool[(uint64_t)i * cap + fwd[(uint64_t)i * PK + t]];
        const uint32_t pos = t + min(t, m);
        gi[pos] = kcna_key_id(key);
        gd[pos] = kcna_key_dist(key);
    }
    for (uint32_t t = tid; t < need; t += CG_THREADS) {
        const uint32_t src = (uint32_t)(s[t] & 0xFFFFFFFFull);
        const uint32_t pos = min(t + 1, nk) + t;
        gi[pos] = src;
        gd[pos] = rows_l2(rows, i, src);
    }
    for (uint32_t p = deg + tid; p < W; p += CG_THREADS) gi[p] = 0xFFFFFFFFu;
    if (tid == 0) g_deg[i] = deg;
}

} // namespace

kcna_status kcna_cagra_prune(kcna_ctx *c, const kcna_params *p) {
    if (!c->has_pools) return kcna_fail(c, KCNA_E_STATE, "prune: no pools (run NN-descent or set pools first)");
    const uint32_t K = p->K, PK = K / 2, N = c->n;
    if (K < 2 || K > c->cap || K > 1024)
        return kcna_fail(c, KCNA_E_ARG, "CAGRA prune: K must be in [2, min(pool capacity, 1024)]");
    KCNA_TRY(kcna_graph_alloc(c, std::max<uint32_t>(c->W, PK + 1)));
    uint32_t P2 = 1;
    while (P2 < K) P2 <<= 1;
    uint16_t *fwd = nullptr;
    uint32_t *indeg = nullptr, *cursor = nullptr;
    uint64_t *off = nullptr, *rev = nullptr;
    kcna_status s = KCNA_OK;
    auto cleanup = [&]() {
        kcna_release(c, fwd);
        kcna_release(c, indeg);
        kcna_release(c, cursor);
        kcna_release(c, off);
        kcna_release(c, rev);
    };
    if ((s = kcna_alloc(c, &fwd, (uint64_t)N * PK, "CAGRA kept ranks")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &indeg, N, "CAGRA in-degrees")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &cursor, N, "CAGRA cursors")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &off, (uint64_t)N + 1, "CAGRA offsets")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_phase_begin(c)) != KCNA_OK) return cleanup(), s;
    cudaMemsetAsync(indeg, 0, (size_t)N * 4, c->stream);
    cudaMemsetAsync(cursor, 0, (size_t)N * 4, c->stream);
    const size_t sm = (size_t)P2 * 8 + (size_t)K * 8 + (size_t)P2 * 16;
    if ((s = kcna_cuda_check(c, cudaFuncSetAttribute(cagra_route_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "cagra smem attr")) != KCNA_OK)
        return cleanup(), s;
    cagra_route_kernel<<<N, CG_THREADS, sm, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, K, PK, P2, fwd, indeg,
                                                         c->d_err);
    KCNA_LAUNCHED(c);
    uint64_t E = 0;
    if ((s = kcna_exclusive_scan_u32(c, indeg, N, off, &E)) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &rev, std::max<uint64_t>(E, 1), "CAGRA reverse entries")) != KCNA_OK) return cleanup(), s;
    cagra_rev_fill_kernel<<<kcna_div_up((uint64_t)N * PK, 256), 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N,
                                                                                      K, PK, fwd, off, cursor, rev);
    KCNA_LAUNCHED(c);
    if (c->bf16_exact)
        cagra_merge_kernel<<<N, CG_THREADS, 0, c->stream>>>(RowsB16{c->Xh, (int)c->ld}, c->pool, c->pool_cnt, c->cap,
                                                            N, K, PK, fwd, off, rev, c->g_ids, c->g_dist, c->g_deg,
                                                            c->W, c->d_err);
    else
        cagra_merge_kernel<<<N, CG_THREADS, 0, c->stream>>>(RowsF32{c->X, (int)c->ld}, c->pool, c->pool_cnt, c->cap,
                                                            N, K, PK, fwd, off, rev, c->g_ids, c->g_dist, c->g_deg,
                                                            c->W, c->d_err);
    KCNA_LAUNCHED(c);
    s = kcna_cuda_check(c, cudaGetLastError(), "CAGRA kernels");
    if (s == KCNA_OK) s = kcna_phase_end(c, KCNA_PHASE_PRUNE);
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "CAGRA sync");
    cleanup();
    if (s == KCNA_OK) c->has_graph = true;
    return s;
}
