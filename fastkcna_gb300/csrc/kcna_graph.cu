// kcna_graph.cu - occlusion prune, link, entry point, connectivity, P2K
// refinement and beam search on the GPU.
//
// Reference functions replaced (src/kgraph.cpp):
//   nsg_sync_prune :1809-1851, taumg_sync_prune :2833-2876,
//   alphapg_sync_prune :3157-3203          -> prune_kernel (warp per node)
//   InterInsert :2051-2084 + *_reversed_prune :2012-2048/:3038-3083/:3374-3422
//   inside nsg_Link :2087-2143 (and the tau / angle twins) -> link kernels
//   ComputeEp :1528-1536, Calcenter (src/kgraph-data.h:413-428),
//   get_neighbors :1560-1623               -> centroid + beam_search_kernel
//   tree_grow :2145-2172, findroot :2174-2236, DFS :2238-2270 -> BFS + attach
//   UpdateNhoods :3537-3584                -> update_nhoods_kernel
//   BridgeView :2478-2663                  -> bridge_* kernels + the shared merge
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <random>
#include <set>

#include "kcna_internal.h"
#include "kcna_sort.cuh"

namespace {

struct PruneRule {
    int kind;
    float t3;  // 3 * tau (FP32, src/kgraph.cpp:2859)
    float thr; // cos(angle) as the reference computes it (src/kgraph.cpp:3161)
};

// Occlusion of candidate p (distance pd to the node) by kept t (distance td to
// the node) at distance djk between them.
__device__ __forceinline__ bool occludes(const PruneRule &r, float td, float djk, float pd) {
    if (r.kind == KCNA_TAUMNG) return djk < __fsub_rn(pd, r.t3);
    if (r.kind == KCNA_ALPHAPG) {
        float num = __fdiv_rn(__fsub_rn(__fadd_rn(td, djk), pd), 2.0f);
        float cs = __fdiv_rn(num, __fsqrt_rn(__fmul_rn(td, djk)));
        return djk < pd && cs < r.thr;
    }
    return djk < pd;
}

// Occlusion prune of one candidate list by one warp, in the reference's order
// (kept[0] = first candidate; each later candidate p is dropped when a kept t
// has the same id or occludes it; stop at `range` kept), with the same result
// as the sequential scan.  Almost every candidate is occluded by one of the
// first kept neighbours, so each batch of 32 candidates (one per lane) is first
// tested against kept[0..3] with four independent FMA chains (the candidate row
// is read once, eight loads in flight); the few survivors are then tested one
// at a time against kept[4..nk) with one lane per kept row; finally the batch
// is resolved in candidate order (the first unoccluded lane is kept and tests
// the later lanes).  Rows are read through R (FP32 or exact BF16 copy).
// With nk0 > 0 the scan continues a kept list kid/kd[0, nk0) (from a prune
// that covered the candidates before `first`) at candidate `first`.
template <class R, typename GetFn>
__device__ int warp_prune(const R &rows, uint32_t n_oracle, const PruneRule &rule, int first, int lim, int range,
                          GetFn get, uint32_t *kid, float *kd, unsigned long long *comps, int nk0 = 0) {
    const int lane = kcna_lane();
    const int nv = rows.ld >> 2;
    if (range <= 0) return 0;
    if (first >= lim) return nk0;
    int nk = nk0, start = first;
    if (nk0 == 0) {
        uint32_t id0;
        float d0;
        get(first, id0, d0);
        if (lane == 0) {
            kid[0] = id0;
            kd[0] = d0;
        }
        nk = 1;
        start = first + 1;
    }
    __syncwarp();
    unsigned long long cc = 0;
    for (int base = start; base < lim && nk < range; base += 32) {
        const int i = base + lane;
        uint32_t id = KCNA_NONE;
        float pd = 0.f;
        bool live = false;
        if (i < lim) {
            get(i, id, pd);
            live = id < n_oracle; // src/kgraph.cpp:1822 `if (p.id >= oracle.size()) continue;`
        }
        bool occ = false;
        // phase 1: kept[0..min(nk,4)), four independent chains, candidate row read once
        const int t1 = min(nk, 4);
        if (live) {
            const uint32_t k0 = kid[0], k1 = kid[t1 > 1 ? 1 : 0], k2 = kid[t1 > 2 ? 2 : 0], k3 = kid[t1 > 3 ? 3 : 0];
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
            for (int b0 = 0; b0 < nv; b0 += 8) {
                float4 pv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) pv[u] = b0 + u < nv ? rows.ld4(id, b0 + u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (b0 + u >= nv) break;
                    const int k = b0 + u;
                    a0 = kcna_acc4(a0, rows.ld4(k0, k), pv[u]);
                    if (t1 > 1) a1 = kcna_acc4(a1, rows.ld4(k1, k), pv[u]);
                    if (t1 > 2) a2 = kcna_acc4(a2, rows.ld4(k2, k), pv[u]);
                    if (t1 > 3) a3 = kcna_acc4(a3, rows.ld4(k3, k), pv[u]);
                }
            }
            const float ds[4] = {a0, a1, a2, a3};
            for (int t = 0; t < t1; ++t) {
                if (kid[t] == id) {
                    occ = true;
                    break;
                }
                ++cc;
                if (occludes(rule, kd[t], ds[t], pd)) {
                    occ = true;
                    break;
                }
            }
        }
        unsigned rem = __ballot_sync(KCNA_FULL, live && !occ);
        // phase 2: survivors against kept[4..nk), one lane per kept row
        if (nk > 4) {
            unsigned todo = rem;
            while (todo) {
                const int b = __ffs(todo) - 1;
                todo &= todo - 1;
                const uint32_t bid = __shfl_sync(KCNA_FULL, id, b);
                const float bd = __shfl_sync(KCNA_FULL, pd, b);
                bool hit = false;
                for (int t0 = 4; t0 < nk && !hit; t0 += 32) {
                    const int t = t0 + lane;
                    bool h = false;
                    if (t < nk) {
                        if (kid[t] == bid) {
                            h = true;
                        } else {
                            ++cc;
                            h = occludes(rule, kd[t], rows_l2(rows, kid[t], bid), bd);
                        }
                    }
                    hit = __ballot_sync(KCNA_FULL, h) != 0;
                }
                if (hit) rem &= ~(1u << b);
            }
        }
        // in-batch resolution, in candidate order
        while (rem && nk < range) {
            const int a = __ffs(rem) - 1;
            const uint32_t aid = __shfl_sync(KCNA_FULL, id, a);
            const float ad = __shfl_sync(KCNA_FULL, pd, a);
            if (lane == 0) {
                kid[nk] = aid;
                kd[nk] = ad;
            }
            ++nk;
            __syncwarp();
            rem &= ~((2u << a) - 1u); // lanes after a
            const bool mine = (rem >> lane) & 1u;
            bool o2 = false;
            if (mine) {
                if (aid == id) {
                    o2 = true;
                } else {
                    ++cc;
                    o2 = occludes(rule, ad, rows_l2(rows, aid, id), pd);
                }
            }
            rem &= ~__ballot_sync(KCNA_FULL, o2);
        }
    }
    cc = kcna_warp_sum(cc);
    if (lane == 0 && comps && cc) atomicAdd(comps, cc);
    __syncwarp();
    return nk;
}

constexpr int PW = 4; // warps per prune block

template <class R>
__global__ void __launch_bounds__(PW * 32) prune_kernel(R rows, uint32_t N, const uint64_t *__restrict__ pool,
                                                        const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                                        PruneRule rule, int range, int maxc,
                                                        uint32_t *__restrict__ g_ids, float *__restrict__ g_dist,
                                                        uint32_t *__restrict__ g_deg, uint32_t W,
                                                        unsigned long long *comps, uint32_t n_items,
                                                        const uint32_t *__restrict__ list) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    uint32_t *kid = reinterpret_cast<uint32_t *>(smem) + w * 2 * range;
    float *kd = reinterpret_cast<float *>(kid + range);
    const uint32_t item = blockIdx.x * PW + w; // node, or the item-th node of `list`
    if (item >= n_items) return;
    const uint32_t q = list ? list[item] : item;
    const uint64_t *pr = pool + (uint64_t)q * cap;
    const int cnt = (int)pool_cnt[q];
    int first = 0;
    if (cnt > 0 && kcna_key_id(pr[0]) == q) first = 1;
    const int lim = min(cnt, maxc);
    auto get = [&](int i, uint32_t &id, float &dd) {
        uint64_t k = pr[i];
        id = kcna_key_id(k);
        dd = kcna_key_dist(k);
    };
    const int nk = (first < cnt) ? warp_prune(rows, N, rule, first, max(lim, first + 1), range, get, kid, kd, comps) : 0;
    for (int j = lane; j < (int)W; j += 32) {
        g_ids[(uint64_t)q * W + j] = j < nk ? kid[j] : KCNA_NONE;
        g_dist[(uint64_t)q * W + j] = j < nk ? kd[j] : 0.f;
    }
    if (lane == 0) g_deg[q] = nk;
}

// Finishes the prunes a screened tile prune left at the end of its tile
// (kcna_prune_fp8.cu): each listed item continues its node's kept list g_ids
// / g_dist[0, g_deg) with the FP32 warp prune from candidate `skip` after the
// first, the same scan as prune_kernel.  Items index the candidate rows of
// `keys` (`stride` apart, cnt[row] candidates); with `nodes` the row of item
// k is k and its node nodes[k] (the link's staged lists), else both are k
// (the pools).
template <class R>
__global__ void __launch_bounds__(PW * 32) prune_resume_kernel(R rows, uint32_t n_oracle,
                                                               const uint64_t *__restrict__ keys, uint64_t stride,
                                                               const uint32_t *__restrict__ cnts,
                                                               const uint32_t *__restrict__ nodes, PruneRule rule,
                                                               int range, int maxc, int skip,
                                                               const uint32_t *__restrict__ list,
                                                               const uint32_t *__restrict__ list_cnt,
                                                               uint32_t *__restrict__ g_ids, float *__restrict__ g_dist,
                                                               uint32_t *__restrict__ g_deg, uint32_t W,
                                                               unsigned long long *comps) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    uint32_t *kid = reinterpret_cast<uint32_t *>(smem) + w * 2 * range;
    float *kd = reinterpret_cast<float *>(kid + range);
    const uint32_t nl = *list_cnt;
    for (uint32_t i = blockIdx.x * PW + w; i < nl; i += gridDim.x * PW) {
        const uint32_t item = list[i];
        const uint32_t q = nodes ? nodes[item] : item;
        const uint64_t *pr = keys + (uint64_t)item * stride;
        const int cnt = (int)cnts[item];
        const int first = cnt > 0 && kcna_key_id(pr[0]) == q ? 1 : 0;
        const int lim = max(min(cnt, maxc), first + 1);
        const int nk0 = (int)min(g_deg[q], (uint32_t)range);
        for (int j = lane; j < nk0; j += 32) {
            kid[j] = g_ids[(uint64_t)q * W + j];
            kd[j] = g_dist[(uint64_t)q * W + j];
        }
        __syncwarp();
        auto get = [&](int i2, uint32_t &id, float &dd) {
            const uint64_t k = pr[i2];
            id = kcna_key_id(k);
            dd = kcna_key_dist(k);
        };
        const int nk = nk0 > 0 ? warp_prune(rows, n_oracle, rule, first + skip, lim, range, get, kid, kd, comps, nk0) : 0;
        for (int j = lane; j < (int)W; j += 32) {
            g_ids[(uint64_t)q * W + j] = j < nk ? kid[j] : KCNA_NONE;
            g_dist[(uint64_t)q * W + j] = j < nk ? kd[j] : 0.f;
        }
        if (lane == 0) g_deg[q] = (uint32_t)nk;
        __syncwarp();
    }
}

// ---- link: reverse edges -------------------------------------------------
__global__ void rev_count_kernel(const uint32_t *__restrict__ g_ids, const uint32_t *__restrict__ g_deg, uint32_t N,
                                 uint32_t W, uint32_t *__restrict__ indeg) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)N * W) return;
    uint32_t n = (uint32_t)(t / W), j = (uint32_t)(t % W);
    if (j >= g_deg[n]) return;
    uint32_t des = g_ids[t];
    if (des < N) atomicAdd(indeg + des, 1u);
}
// Reverse edge n -> des as (n << 32 | distance bits): the distance of the
// kept edge is the canonical d(n, des), equal bit for bit to d(des, n), so
// InterInsert needs no distance evaluation.
__global__ void rev_fill_kernel(const uint32_t *__restrict__ g_ids, const float *__restrict__ g_dist,
                                const uint32_t *__restrict__ g_deg, uint32_t N, uint32_t W,
                                const uint64_t *__restrict__ off, uint32_t *__restrict__ cursor,
                                uint64_t *__restrict__ rev) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)N * W) return;
    uint32_t n = (uint32_t)(t / W), j = (uint32_t)(t % W);
    if (j >= g_deg[n]) return;
    uint32_t des = g_ids[t];
    if (des >= N) return;
    uint32_t p = atomicAdd(cursor + des, 1u);
    rev[off[des] + p] = ((uint64_t)n << 32) | __float_as_uint(g_dist[t]);
}

// exclusive scan of u32 counts into u64 offsets (3 phases)
constexpr int SCAN_T = 1024, SCAN_E = 4;
__global__ void scan_block_sums(const uint32_t *__restrict__ in, uint64_t n, uint64_t *__restrict__ sums) {
    __shared__ uint64_t s[SCAN_T / 32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_T * SCAN_E;
    uint64_t v = 0;
    for (int e = 0; e < SCAN_E; ++e) {
        uint64_t i = base + (uint64_t)e * SCAN_T + threadIdx.x;
        if (i < n) v += in[i];
    }
    v = kcna_warp_sum(v);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int i = 0; i < SCAN_T / 32; ++i) t += s[i];
        sums[blockIdx.x] = t;
    }
}
__global__ void scan_sums_serial(uint64_t *sums, uint32_t nb, uint64_t *total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint64_t run = 0;
    for (uint32_t i = 0; i < nb; ++i) {
        uint64_t t = sums[i];
        sums[i] = run;
        run += t;
    }
    *total = run;
}
__global__ void scan_apply(const uint32_t *__restrict__ in, uint64_t n, const uint64_t *__restrict__ sums,
                           uint64_t *__restrict__ out) {
    __shared__ uint64_t s[SCAN_T];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_T * SCAN_E;
    uint64_t run = sums[blockIdx.x];
    for (int e = 0; e < SCAN_E; ++e) {
        uint64_t i = base + (uint64_t)e * SCAN_T + threadIdx.x;
        uint64_t v = i < n ? in[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_T; o <<= 1) {
            uint64_t u = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += u;
            __syncthreads();
        }
        if (i < n) out[i] = run + s[threadIdx.x] - v;
        uint64_t tot = s[SCAN_T - 1];
        __syncthreads();
        run += tot;
    }
}

// Per node: pruned list + reverse sources (sorted by id, not already present),
// then the reversed prune when the list exceeds range.
constexpr int LT = 128;
constexpr int LCAP = 4096; // merged-list capacity per node in shared memory

template <class R>
__global__ void __launch_bounds__(LT) link_merge_kernel(R rows, uint32_t N, PruneRule rule, int range,
                                                       uint32_t *__restrict__ g_ids, float *__restrict__ g_dist,
                                                       uint32_t *__restrict__ g_deg, uint32_t W,
                                                       const uint64_t *__restrict__ off,
                                                       const uint64_t *__restrict__ rev,
                                                       unsigned long long *comps, int *err,
                                                       const uint32_t *__restrict__ nodes) {
    __shared__ uint64_t s_key[LCAP];   // sorting keys (rev (id, dist); later (dist, position))
    __shared__ uint32_t s_id[LCAP];
    __shared__ float s_d[LCAP];
    __shared__ uint32_t s_kid[128];
    __shared__ float s_kd[128];
    __shared__ uint32_t s_warp[LT / 32];
    __shared__ int s_nk;
    const uint32_t q = nodes ? nodes[blockIdx.x] : blockIdx.x;
    const int deg = (int)g_deg[q];
    const uint64_t r0 = off[q], r1 = off[q + 1];
    const uint64_t room = (uint64_t)(LCAP - deg);
    int nin = (int)((r1 - r0) < room ? (r1 - r0) : room);
    if ((uint64_t)nin < r1 - r0) kcna_set_err(err, KCNA_DERR_BOUNDS);
    // pruned entries first, in order
    for (int j = threadIdx.x; j < deg; j += LT) {
        s_id[j] = g_ids[(uint64_t)q * W + j];
        s_d[j] = g_dist[(uint64_t)q * W + j];
    }
    // reverse sources sorted by id (each with its distance in the low word)
    const int np2 = kcna_pow2_ceil_d(max(nin, 1));
    for (int j = threadIdx.x; j < np2; j += LT) s_key[j] = j < nin ? rev[r0 + j] : KCNA_EMPTY_KEY;
    kcna_cta_bitonic(s_key, np2);
    // keep sources not in the pruned list (InterInsert dup check, :2064-2071)
    int keep_local = 0;
    const int per = (nin + LT - 1) / LT;
    const int b = threadIdx.x * per;
    uint32_t flags = 0;
    for (int e = 0; e < per && b + e < nin; ++e) {
        uint32_t src = (uint32_t)(s_key[b + e] >> 32);
        bool dup = false;
        for (int j = 0; j < deg; ++j)
            if (s_id[j] == src) {
                dup = true;
                break;
            }
        if (!dup) {
            flags |= 1u << e;
            ++keep_local;
        }
    }
    // block exclusive scan of keep counts
    int incl = keep_local;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(KCNA_FULL, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < LT / 32; ++i) {
            uint32_t t = s_warp[i];
            s_warp[i] = run;
            run += t;
        }
        s_nk = (int)run;
    }
    __syncthreads();
    int pos = deg + (int)s_warp[w] + incl - keep_local;
    for (int e = 0; e < per && b + e < nin; ++e)
        if (flags & (1u << e)) {
            s_id[pos] = (uint32_t)(s_key[b + e] >> 32);
            s_d[pos] = __uint_as_float((uint32_t)s_key[b + e]); // oracle(n, des), from the reverse edge
            ++pos;
        }
    const int total = deg + s_nk;
    __syncthreads();
    if (total <= range) {
        for (int j = threadIdx.x; j < (int)W; j += LT) {
            g_ids[(uint64_t)q * W + j] = j < total ? s_id[j] : KCNA_NONE;
            g_dist[(uint64_t)q * W + j] = j < total ? s_d[j] : 0.f;
        }
        if (threadIdx.x == 0) g_deg[q] = total;
        return;
    }
    // reversed prune: stable sort by distance, then the occlusion scan without the search_K cap
    const int tp = kcna_pow2_ceil_d(total);
    for (int j = threadIdx.x; j < tp; j += LT)
        s_key[j] = j < total ? (((uint64_t)__float_as_uint(s_d[j]) << 32) | (uint32_t)j) : KCNA_EMPTY_KEY;
    kcna_cta_bitonic(s_key, tp);
    if (threadIdx.x < 32) {
        auto get = [&](int i, uint32_t &id, float &dd) {
            uint32_t p = (uint32_t)s_key[i];
            id = s_id[p];
            dd = s_d[p];
        };
        int first = 0;
        {
            uint32_t id0;
            float d0;
            get(0, id0, d0);
            if (id0 == q) first = 1;
        }
        int nk = warp_prune(rows, 0xFFFFFFFFu, rule, first, total, range, get, s_kid, s_kd, comps);
        for (int j = lane; j < (int)W; j += 32) {
            g_ids[(uint64_t)q * W + j] = j < nk ? s_kid[j] : KCNA_NONE;
            g_dist[(uint64_t)q * W + j] = j < nk ? s_kd[j] : 0.f;
        }
        if (lane == 0) g_deg[q] = nk;
    }
}

// Warp per node, persistent: the same InterInsert merge and reversed prune as
// link_merge_kernel for the common node whose pruned list and reverse
// sources fit LW_CAP entries; larger nodes are queued for the block kernel.
constexpr int LW_WARPS = 4, LW_CAP = 256;

template <class R>
__global__ void __launch_bounds__(LW_WARPS * 32) link_warp_kernel(R rows, uint32_t N, PruneRule rule, int range,
                                                                 uint32_t *__restrict__ g_ids,
                                                                 float *__restrict__ g_dist,
                                                                 uint32_t *__restrict__ g_deg, uint32_t W,
                                                                 const uint64_t *__restrict__ off,
                                                                 const uint64_t *__restrict__ rev,
                                                                 unsigned long long *comps, uint32_t *big_list,
                                                                 uint32_t *big_cnt, uint64_t *stage,
                                                                 uint32_t *stage_nodes, uint32_t *stage_cnt,
                                                                 uint32_t *stage_n) {
    __shared__ uint64_t s_key[LW_WARPS][LW_CAP];
    __shared__ uint32_t s_id[LW_WARPS][LW_CAP];
    __shared__ float s_d[LW_WARPS][LW_CAP];
    __shared__ uint32_t s_kid[LW_WARPS][128];
    __shared__ float s_kd[LW_WARPS][128];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    uint64_t *key = s_key[w];
    uint32_t *ids = s_id[w];
    float *ds = s_d[w];
    for (uint32_t q = blockIdx.x * LW_WARPS + w; q < N; q += gridDim.x * LW_WARPS) {
        const int deg = (int)min(g_deg[q], W);
        const uint64_t r0 = off[q], r1 = off[q + 1];
        const int nin = (int)(r1 - r0);
        if (deg + nin > LW_CAP) {
            if (lane == 0) big_list[atomicAdd(big_cnt, 1u)] = q;
            continue;
        }
        for (int j = lane; j < deg; j += 32) {
            ids[j] = g_ids[(uint64_t)q * W + j];
            ds[j] = g_dist[(uint64_t)q * W + j];
        }
        // reverse sources (id << 32 | distance) sorted by id
        const int np2 = kcna_pow2_ceil_d(max(nin, 1));
        for (int j = lane; j < np2; j += 32) key[j] = j < nin ? rev[r0 + j] : KCNA_EMPTY_KEY;
        kcna_warp_bitonic(key, np2);
        // sources not in the pruned list, appended in id order (InterInsert, :2064-2071)
        int total = deg;
        for (int b0 = 0; b0 < nin; b0 += 32) {
            const int j = b0 + lane;
            bool keep = false;
            uint64_t k = 0;
            if (j < nin) {
                k = key[j];
                const uint32_t src = (uint32_t)(k >> 32);
                keep = true;
                for (int t = 0; t < deg; ++t)
                    if (ids[t] == src) {
                        keep = false;
                        break;
                    }
            }
            const unsigned m = __ballot_sync(KCNA_FULL, keep);
            if (keep) {
                const int pos = total + __popc(m & kcna_lanemask_lt());
                ids[pos] = (uint32_t)(k >> 32);
                ds[pos] = __uint_as_float((uint32_t)k); // oracle(n, des), from the reverse edge
            }
            total += __popc(m);
        }
        __syncwarp();
        uint32_t *gi = g_ids + (uint64_t)q * W;
        float *gd = g_dist + (uint64_t)q * W;
        if (total <= range) {
            for (int j = lane; j < (int)W; j += 32) {
                gi[j] = j < total ? ids[j] : KCNA_NONE;
                gd[j] = j < total ? ds[j] : 0.f;
            }
            if (lane == 0) g_deg[q] = (uint32_t)total;
            continue;
        }
        // reversed prune: stable sort by distance, then the occlusion scan without the search_K cap
        const int tp = kcna_pow2_ceil_d(total);
        for (int j = lane; j < tp; j += 32)
            key[j] = j < total ? (((uint64_t)__float_as_uint(ds[j]) << 32) | (uint32_t)j) : KCNA_EMPTY_KEY;
        kcna_warp_bitonic(key, tp);
        if (stage) { // the FP8-screened tile prune takes the list (pool-format keys, LW_CAP apart)
            uint32_t slot = 0;
            if (lane == 0) slot = atomicAdd(stage_n, 1u);
            slot = __shfl_sync(KCNA_FULL, slot, 0);
            uint64_t *dst = stage + (uint64_t)slot * LW_CAP;
            for (int j = lane; j < total; j += 32) {
                const uint32_t p = (uint32_t)key[j];
                dst[j] = ((uint64_t)__float_as_uint(ds[p]) << 32) | ((uint64_t)ids[p] << 2);
            }
            if (lane == 0) {
                stage_nodes[slot] = q;
                stage_cnt[slot] = (uint32_t)total;
            }
            __syncwarp();
            continue;
        }
        auto get = [&](int i, uint32_t &id, float &dd) {
            const uint32_t p = (uint32_t)key[i];
            id = ids[p];
            dd = ds[p];
        };
        const int first = ids[(uint32_t)key[0]] == q ? 1 : 0;
        const int nk = warp_prune(rows, 0xFFFFFFFFu, rule, first, total, range, get, s_kid[w], s_kd[w], comps);
        for (int j = lane; j < (int)W; j += 32) {
            gi[j] = j < nk ? s_kid[w][j] : KCNA_NONE;
            gd[j] = j < nk ? s_kd[w][j] : 0.f;
        }
        if (lane == 0) g_deg[q] = (uint32_t)nk;
        __syncwarp();
    }
}

// ---- entry point: centroid + beam search --------------------------------
constexpr int CB_ROWS = 1024;
__global__ void centroid_partial_kernel(const float *__restrict__ X, int ld, uint32_t n, int d,
                                        double *__restrict__ part) {
    const uint32_t r0 = blockIdx.x * CB_ROWS, r1 = min(n, r0 + CB_ROWS);
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
        double s = 0;
        for (uint32_t r = r0; r < r1; ++r) s += X[(uint64_t)r * ld + j];
        part[(uint64_t)blockIdx.x * d + j] = s;
    }
}
__global__ void centroid_final_kernel(const double *__restrict__ part, uint32_t nb, int d, int ld, uint32_t n,
                                      float *__restrict__ center) {
    for (int j = threadIdx.x; j < ld; j += blockDim.x) {
        double s = 0;
        for (uint32_t b = 0; b < nb; ++b) s += j < d ? part[(uint64_t)b * d + j] : 0.0;
        center[j] = j < d ? (float)(s / n) : 0.f;
    }
}

// Beam search of one query per warp (get_neighbors semantics).  Pool of L+1
// keys in shared memory; bit 0 of a key = not yet expanded.  visited: one
// bitmap of N bits per resident warp slot in global memory.
constexpr int BW = 4;

// InsertIntoPool (src/kgraph.cpp:261-298) on keys ordered by distance only.
__device__ int pool_insert_pos(const uint64_t *pool, int K, float dist, uint32_t id) {
    int left = 0, right = K - 1;
    if (kcna_key_dist(pool[left]) > dist) return -1; // insert at 0
    if (kcna_key_dist(pool[right]) < dist) return K; // append
    while (left < right - 1) {
        int mid = (left + right) / 2;
        if (kcna_key_dist(pool[mid]) > dist)
            right = mid;
        else
            left = mid;
    }
    while (left > 0) {
        if (kcna_key_dist(pool[left]) < dist) break;
        if (kcna_key_id(pool[left]) == id) return K + 1;
        left--;
    }
    if (kcna_key_id(pool[left]) == id || kcna_key_id(pool[right]) == id) return K + 1;
    return right;
}

__global__ void __launch_bounds__(BW * 32) beam_search_kernel(const float *__restrict__ X, int ld, uint32_t N,
                                                              const uint32_t *__restrict__ g_ids,
                                                              const uint32_t *__restrict__ g_deg, uint32_t W,
                                                              const float *__restrict__ Q, uint32_t m,
                                                              const uint32_t *__restrict__ init_ids, int L, int k,
                                                              uint32_t *__restrict__ visited, uint32_t vwords,
                                                              uint32_t *__restrict__ out_ids,
                                                              float *__restrict__ out_d) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = kcna_lane();
    uint64_t *pool = reinterpret_cast<uint64_t *>(smem) + (uint64_t)w * (L + 1);
    const uint32_t slot = blockIdx.x * BW + w;
    uint32_t *vis = visited + (uint64_t)slot * vwords;
    const uint32_t nslots = gridDim.x * BW;
    for (uint32_t qi = slot; qi < m; qi += nslots) {
        for (uint32_t i = lane; i < vwords; i += 32) vis[i] = 0;
        __syncwarp();
        const float *qrow = Q + (uint64_t)qi * ld;
        const uint32_t *init = init_ids + (uint64_t)qi * L;
        // init: mark, compute, sort
        for (int i = lane; i < L; i += 32) {
            uint32_t id = init[i];
            if (id < N) atomicOr(vis + (id >> 5), 1u << (id & 31));
        }
        __syncwarp();
        int Lc = 0;
        for (int b0 = 0; b0 < L; b0 += 32) {
            int i = b0 + lane;
            uint32_t id = i < L ? init[i] : KCNA_NONE;
            bool ok = id < N;
            uint64_t key = KCNA_EMPTY_KEY;
            if (ok) key = kcna_key(kcna_l2_ldg(qrow, X + (uint64_t)id * ld, ld), id, 1u);
            unsigned mk = __ballot_sync(KCNA_FULL, ok);
            if (ok) pool[Lc + __popc(mk & kcna_lanemask_lt())] = key;
            Lc += __popc(mk);
        }
        const int p2 = kcna_pow2_ceil_d(max(Lc, 1));
        // sort pool[0..Lc) (pad into the free slots beyond L with care: use a local sort)
        if (p2 <= L + 1) {
            for (int i = Lc + lane; i < p2; i += 32) pool[i] = KCNA_EMPTY_KEY;
            kcna_warp_bitonic(pool, p2);
        } else if (lane == 0) { // insertion sort (Lc > (L+1)/2 and not a power of two)
            for (int i = 1; i < Lc; ++i) {
                uint64_t v = pool[i];
                int j = i - 1;
                while (j >= 0 && pool[j] > v) {
                    pool[j + 1] = pool[j];
                    --j;
                }
                pool[j + 1] = v;
            }
        }
        __syncwarp();
        int kk = 0;
        while (kk < Lc) {
            int nk = Lc;
            uint64_t cur = pool[kk];
            if (cur & 1ull) {
                __syncwarp();
                if (lane == 0) pool[kk] = cur & ~1ull;
                __syncwarp();
                const uint32_t nid = kcna_key_id(cur);
                const int deg = (int)min(g_deg[nid], W);
                for (int b0 = 0; b0 < deg; b0 += 32) {
                    int j = b0 + lane;
                    uint32_t id = j < deg ? g_ids[(uint64_t)nid * W + j] : KCNA_NONE;
                    bool fresh = false;
                    if (id < N) {
                        uint32_t old = atomicOr(vis + (id >> 5), 1u << (id & 31));
                        fresh = !(old & (1u << (id & 31)));
                    }
                    float dist = fresh ? kcna_l2_ldg(qrow, X + (uint64_t)id * ld, ld) : 0.f;
                    unsigned mk = __ballot_sync(KCNA_FULL, fresh);
                    // apply in neighbour order, as the reference does
                    while (mk) {
                        int src = __ffs(mk) - 1;
                        mk &= mk - 1;
                        uint32_t cid = __shfl_sync(KCNA_FULL, id, src);
                        float cd = __shfl_sync(KCNA_FULL, dist, src);
                        if (cd >= kcna_key_dist(pool[Lc - 1])) continue;
                        int r = 0;
                        if (lane == 0) r = pool_insert_pos(pool, Lc, cd, cid);
                        r = __shfl_sync(KCNA_FULL, r, 0);
                        if (r == Lc + 1) continue; // duplicate: InsertIntoPool returns K+1, L still grows below
                        int at = r < 0 ? 0 : r;
                        __syncwarp();
                        if (lane == 0) {
                            for (int t = Lc; t > at; --t) pool[t] = pool[t - 1];
                            pool[at] = kcna_key(cd, cid, 1u);
                        }
                        __syncwarp();
                        if (Lc < L) ++Lc;
                        if (at < nk) nk = at;
                    }
                }
            }
            if (nk <= kk)
                kk = nk;
            else
                ++kk;
        }
        for (int i = lane; i < k; i += 32) {
            uint64_t key = i < Lc ? pool[i] : KCNA_EMPTY_KEY;
            out_ids[(uint64_t)qi * k + i] = i < Lc ? kcna_key_id(key) : KCNA_NONE;
            out_d[(uint64_t)qi * k + i] = i < Lc ? kcna_key_dist(key) : __uint_as_float(0x7F800000u);
        }
        __syncwarp();
    }
}

// ---- tree_grow: BFS reachability + attach --------------------------------
__global__ void bfs_expand_kernel(const uint32_t *__restrict__ g_ids, const uint32_t *__restrict__ g_deg, uint32_t W,
                                  uint32_t N, const uint32_t *__restrict__ frontier, uint32_t nf,
                                  uint32_t *__restrict__ visited, uint32_t *__restrict__ next,
                                  uint32_t *__restrict__ next_cnt) {
    const uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (wi >= nf) return;
    const uint32_t u = frontier[wi];
    const int deg = (int)min(g_deg[u], W);
    for (int j = lane; j < deg; j += 32) {
        uint32_t v = g_ids[(uint64_t)u * W + j];
        if (v >= N) continue;
        uint32_t old = atomicOr(visited + (v >> 5), 1u << (v & 31));
        if (!(old & (1u << (v & 31)))) next[atomicAdd(next_cnt, 1u)] = v;
    }
}

// Parallel attach rounds for tree_grow (src/kgraph.cpp:2145-2236).  The
// reference walks unreached ids in order, attaching each not-yet-reached one
// to a reached node and running a DFS from it, so it adds one edge per
// unreached component source.  Here every round attaches all sources at once:
// an unreached node is a source when no unreached node has an edge to it
// (mark_targets_kernel); when every unreached node has such an edge (the rest
// are cycles) the nodes whose id is below all their unreached out-neighbours
// are used.  The attach point is the reference's rule as it runs: findroot
// scans `nhoods[id].pool` with an `id` read in its own initialiser
// (src/kgraph.cpp:2207), which the reference's builds evaluate as 0, so the
// root is the first entry of node 0's pool (over the first pool_cnt[u]
// positions) that is reached and has degree < nsg_R, else a random reached
// node with degree < nsg_R * factor (factor grows when every reached node has
// reached the bound); slots are reserved with atomicAdd on the degree.  As in
// the reference, whose first findroot takes the smallest unreached id, node 0
// is attached first when the entry point does not reach it.  The random
// pick draws from a list of the reached nodes below the bound, rebuilt each
// round (collect_open_kernel), in place of the reference's retries over all
// ids; a node's degree is capped at the graph width W (nsg_R + 8), where the
// reference's list can grow without bound.
__global__ void mark_targets_kernel(const uint32_t *__restrict__ g_ids, const uint32_t *__restrict__ g_deg,
                                    uint32_t W, uint32_t N, const uint32_t *__restrict__ visited,
                                    uint32_t *__restrict__ targeted, uint32_t *__restrict__ localmin,
                                    unsigned long long *n_unreached) {
    const uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (u >= N || ((visited[u >> 5] >> (u & 31)) & 1u)) return;
    const int deg = (int)min(g_deg[u], W);
    bool below_all = true;
    for (int j = lane; j < deg; j += 32) {
        const uint32_t v = g_ids[(uint64_t)u * W + j];
        if (v < N && !((visited[v >> 5] >> (v & 31)) & 1u)) {
            atomicOr(targeted + (v >> 5), 1u << (v & 31));
            if (v < u) below_all = false;
        }
    }
    below_all = __all_sync(KCNA_FULL, below_all);
    if (lane == 0) {
        if (below_all) atomicOr(localmin + (u >> 5), 1u << (u & 31));
        atomicAdd(n_unreached, 1ull);
    }
}

// Reached nodes whose degree is below `limit` (and the width), appended to
// `open` (order irrelevant: picks are random).
__global__ void collect_open_kernel(const uint32_t *__restrict__ visited, const uint32_t *__restrict__ g_deg, uint32_t N,
                                    uint32_t limit, uint32_t W, uint32_t *__restrict__ open, uint32_t *__restrict__ n_open) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = u < N && ((visited[u >> 5] >> (u & 31)) & 1u) && g_deg[u] < limit && g_deg[u] < W;
    const unsigned m = __ballot_sync(KCNA_FULL, ok);
    uint32_t base = 0;
    if (kcna_lane() == 0 && m) base = atomicAdd(n_open, (uint32_t)__popc(m));
    base = __shfl_sync(KCNA_FULL, base, 0);
    if (ok) open[base + __popc(m & kcna_lanemask_lt())] = u;
}

__device__ __forceinline__ bool reserve_slot(uint32_t *g_deg, uint32_t r, uint32_t limit, uint32_t W, uint32_t *slot) {
    const uint32_t old = atomicAdd(g_deg + r, 1u);
    if (old < limit && old < W) {
        *slot = old;
        return true;
    }
    atomicSub(g_deg + r, 1u);
    return false;
}

__global__ void attach_sources_kernel(const float *__restrict__ X, int ld, uint32_t N,
                                      const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                      uint32_t cap, uint32_t *__restrict__ g_ids, float *__restrict__ g_dist,
                                      uint32_t *__restrict__ g_deg, uint32_t W, uint32_t nsg_R,
                                      const uint32_t *__restrict__ visited, const uint32_t *__restrict__ pick,
                                      uint32_t *__restrict__ frontier, uint32_t *__restrict__ nfront, uint64_t seed,
                                      const uint32_t *__restrict__ open, uint32_t n_open, uint32_t open_limit,
                                      int *err, unsigned long long *attached) {
    const uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (u >= N || ((visited[u >> 5] >> (u & 31)) & 1u) || !((pick[u >> 5] >> (u & 31)) & 1u)) return;
    uint32_t root = KCNA_NONE, slot = 0;
    const uint32_t cnt = min(min(pool_cnt[u], pool_cnt[0]), cap);
    for (uint32_t b0 = 0; b0 < cnt && root == KCNA_NONE; b0 += 32) {
        const uint32_t i = b0 + lane;
        uint32_t cid = KCNA_NONE;
        if (i < cnt) {
            cid = kcna_key_id(pool[i]); // node 0's pool
            if (!(cid < N && ((visited[cid >> 5] >> (cid & 31)) & 1u) && g_deg[cid] < nsg_R)) cid = KCNA_NONE;
        }
        unsigned mk = __ballot_sync(KCNA_FULL, cid != KCNA_NONE);
        while (mk && root == KCNA_NONE) { // candidates in pool order; a full slot moves on to the next one
            const int src = __ffs(mk) - 1;
            mk &= mk - 1;
            const uint32_t r = __shfl_sync(KCNA_FULL, cid, src);
            uint32_t got = 0, sl = 0;
            if (lane == 0) got = reserve_slot(g_deg, r, nsg_R, W, &sl) ? 1u : 0u;
            got = __shfl_sync(KCNA_FULL, got, 0);
            if (got) {
                root = r;
                slot = __shfl_sync(KCNA_FULL, sl, 0);
            }
        }
    }
    if (root == KCNA_NONE && lane == 0 && n_open > 0) { // random reached node, src/kgraph.cpp:2216-2230
        for (uint32_t t = 0; t < 64 && root == KCNA_NONE; ++t) {
            const uint32_t rid = open[kcna_rand32(seed, u, t) % n_open];
            if (reserve_slot(g_deg, rid, open_limit, W, &slot)) root = rid;
        }
        // the list's nodes may have been filled by other attaches of this round: walk it once
        const uint32_t o = kcna_rand32(seed, u, 64) % n_open;
        for (uint32_t t = 0; t < n_open && root == KCNA_NONE; ++t) {
            const uint32_t rid = open[(o + t) % n_open];
            if (reserve_slot(g_deg, rid, open_limit, W, &slot)) root = rid;
        }
    }
    if (lane == 0 && root != KCNA_NONE) {
        g_ids[(uint64_t)root * W + slot] = u;
        g_dist[(uint64_t)root * W + slot] = kcna_l2(X + (uint64_t)root * ld, X + (uint64_t)u * ld, ld);
        frontier[atomicAdd(nfront, 1u)] = u;
        atomicAdd(attached, 1ull);
    }
}

__global__ void invert_kernel(uint32_t *__restrict__ w, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = ~w[i];
}
__global__ void mark_frontier_kernel(const uint32_t *__restrict__ f, uint32_t nf, uint32_t *__restrict__ visited) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nf) atomicOr(visited + (f[i] >> 5), 1u << (f[i] & 31));
}

// ---- UpdateNhoods ---------------------------------------------------------
__global__ void update_nhoods_kernel(const uint32_t *__restrict__ g_ids, const uint32_t *__restrict__ g_deg,
                                     uint32_t *__restrict__ g_old, uint32_t *__restrict__ g_old_deg,
                                     uint8_t *__restrict__ g_isnew, uint32_t N, uint32_t W, int first) {
    const uint32_t n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (n >= N) return;
    const uint32_t deg = min(g_deg[n], W), odeg = first ? 0 : min(g_old_deg[n], W);
    const uint32_t *cur = g_ids + (uint64_t)n * W;
    uint32_t *old = g_old + (uint64_t)n * W;
    uint8_t flags[2] = {1, 1};
    uint32_t mine[2] = {KCNA_NONE, KCNA_NONE};
    for (int h = 0; h < 2; ++h) {
        uint32_t j = lane + 32 * h;
        if (j < deg) {
            mine[h] = cur[j];
            bool found = false;
            for (uint32_t t = 0; t < odeg; ++t)
                if (old[t] == mine[h]) {
                    found = true;
                    break;
                }
            flags[h] = (first || !found) ? 1 : 0;
        }
    }
    for (uint32_t j = 64 + lane; j < deg; j += 32) { // rows wider than 64
        uint32_t id = cur[j];
        bool found = false;
        for (uint32_t t = 0; t < odeg; ++t)
            if (old[t] == id) {
                found = true;
                break;
            }
        g_isnew[(uint64_t)n * W + j] = (first || !found) ? 1 : 0;
    }
    __syncwarp();
    for (int h = 0; h < 2; ++h) {
        uint32_t j = lane + 32 * h;
        if (j < deg) g_isnew[(uint64_t)n * W + j] = flags[h];
    }
    __syncwarp();
    for (uint32_t j = lane; j < W; j += 32) old[j] = j < deg ? cur[j] : KCNA_NONE;
    if (lane == 0) g_old_deg[n] = deg;
}

// ---- BridgeView (P2K) -----------------------------------------------------
__global__ void bridge_init_kernel(uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                   uint32_t N, int cur_loop, uint32_t pre_L, uint32_t cur_L) {
    const uint32_t n = blockIdx.x;
    const uint32_t cnt = pool_cnt[n];
    uint64_t *pr = pool + (uint64_t)n * cap;
    for (uint32_t j = threadIdx.x; j < cnt; j += blockDim.x) {
        uint64_t k = pr[j] & ~3ull;
        uint64_t f = pr[j] & KCNA_FLAG_NEW;
        if (cur_loop == 0 || j < pre_L || j >= cur_L)
            k |= KCNA_FLAG_NEW; // flag=true, isnew=false
        else
            k |= KCNA_FLAG_NEW | (f ? KCNA_FLAG_ISNEW : 0ull); // isnew = previous flag
        pr[j] = k;
    }
}

// count (pass 0) or emit (pass 1) the pushes of one update round.  Emitting
// writes each push straight into its target's bucket of rnn (offsets from the
// count pass; the pusher's id with its isnew flag in bit 31) and, with pnew,
// marks targets that receive a new pusher.
__global__ void bridge_update_kernel(uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt, uint32_t cap,
                                     uint32_t N, uint32_t Lp, uint32_t S_, int capped, int emit,
                                     uint32_t *__restrict__ tcount, const uint64_t *__restrict__ off,
                                     uint32_t *__restrict__ cursor, uint32_t *__restrict__ rnn,
                                     uint8_t *__restrict__ pnew) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = kcna_lane();
    if (i >= N) return;
    uint64_t *pr = pool + (uint64_t)i * cap;
    const uint32_t lim = min(Lp, pool_cnt[i]);
    uint32_t taken = 0;
    for (uint32_t b0 = 0; b0 < lim && (!capped || taken < S_); b0 += 32) {
        uint32_t j = b0 + lane;
        uint64_t k = j < lim ? pr[j] : 0;
        bool f = j < lim && (k & KCNA_FLAG_NEW);
        unsigned mk = __ballot_sync(KCNA_FULL, f);
        uint32_t rank = taken + __popc(mk & kcna_lanemask_lt());
        bool take = f && (!capped || rank < S_);
        const uint32_t tgt = kcna_key_id(k);
        if (take && tgt < N) {
            if (!emit) {
                atomicAdd(tcount + tgt, 1u);
            } else {
                const bool isnew = (k & KCNA_FLAG_ISNEW) != 0;
                const uint32_t pos = atomicAdd(cursor + tgt, 1u);
                if (off[tgt] + pos < off[tgt + 1]) rnn[off[tgt] + pos] = i | (isnew ? 0x80000000u : 0u);
                if (pnew && isnew) pnew[tgt] = 1;
                pr[j] = k & ~KCNA_FLAG_NEW;
            }
        }
        taken += __popc(__ballot_sync(KCNA_FULL, take));
    }
}

// per node: graph neighbours whose edge is flagged new (UpdateNhoods); warp per node
__global__ void count_new_edges_kernel(const uint8_t *__restrict__ g_isnew, const uint32_t *__restrict__ g_deg,
                                       uint32_t N, uint32_t W, uint16_t *__restrict__ nnew) {
    const uint32_t q = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = kcna_lane();
    if (q >= N) return;
    const uint32_t deg = min(g_deg[q], W);
    uint32_t n = 0;
    for (uint32_t j0 = 0; j0 < deg; j0 += 32)
        n += __popc(__ballot_sync(KCNA_FULL, j0 + lane < deg && g_isnew[(uint64_t)q * W + j0 + lane]));
    if (lane == 0) nnew[q] = (uint16_t)n;
}

// P2K join, tiled: one block per node q.  Rows = pushers u of q (rnn(q), up to
// 128 per tile), columns = q's graph neighbours w (up to 64), staged through
// shared memory in 32-float chunks; each thread keeps RI x 8 canonical FMA
// accumulators.  Pair (u, w) is skipped when u == w or both are old
// (src/kgraph.cpp:2639-2641); survivors within u's radius become candidates of
// u, written as one run per (q, u) after one atomicAdd.
constexpr int PJT = 256, PJC = 64, PJK = 32, PJP = PJK + 4;

template <int RI, class R>
__device__ void p2k_tile(const R &rows, int ld, uint32_t N, const uint32_t *s_u, const uint8_t *s_unew,
                         int nu, const uint32_t *s_w, const uint8_t *s_wnew, int nw, const float *__restrict__ radius,
                         uint64_t *__restrict__ cand, uint32_t *__restrict__ cand_cnt, uint32_t CB, float *s_As,
                         float *s_Bs, float *s_D, unsigned long long *s_cc) {
    const int tid = threadIdx.x, tx = tid & 7, ty = tid >> 3;
    float acc[RI][8];
#pragma unroll
    for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < ld; k0 += PJK) {
        for (int idx = tid; idx < 32 * RI * (PJK / 4); idx += PJT) {
            int r = idx >> 3, c = (idx & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < nu && k0 + c < ld) v = rows.ld4(s_u[r], (k0 + c) >> 2);
            *reinterpret_cast<float4 *>(s_As + r * PJP + c) = v;
        }
        for (int idx = tid; idx < PJC * (PJK / 4); idx += PJT) {
            int r = idx >> 3, c = (idx & 7) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < nw && k0 + c < ld) v = rows.ld4(s_w[r], (k0 + c) >> 2);
            *reinterpret_cast<float4 *>(s_Bs + r * PJP + c) = v;
        }
        __syncthreads();
        const int kend = min(PJK, ld - k0);
        for (int k = 0; k < kend; k += 4) {
            float4 ra[RI], cb[8];
#pragma unroll
            for (int i = 0; i < RI; ++i) ra[i] = *reinterpret_cast<const float4 *>(s_As + (ty + 32 * i) * PJP + k);
#pragma unroll
            for (int j = 0; j < 8; ++j) cb[j] = *reinterpret_cast<const float4 *>(s_Bs + (tx + 8 * j) * PJP + k);
#pragma unroll
            for (int i = 0; i < RI; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = kcna_acc4(acc[i][j], ra[i], cb[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < RI; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) s_D[(ty + 32 * i) * (PJC + 1) + tx + 8 * j] = acc[i][j];
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    unsigned long long cc = 0;
    for (int i = warp; i < nu; i += PJT / 32) {
        const uint32_t u = s_u[i];
        const bool unew = s_unew[i] != 0;
        const float rad = __ldg(radius + u);
        bool ok[2];
        uint64_t keys[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = lane + 32 * h;
            ok[h] = false;
            if (j < nw && s_w[j] != u && (unew || s_wnew[j])) {
                ++cc;
                float dd = s_D[i * (PJC + 1) + j];
                if (dd <= rad) {
                    ok[h] = true;
                    keys[h] = kcna_key(dd, s_w[j], (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
                }
            }
        }
        unsigned m0 = __ballot_sync(KCNA_FULL, ok[0]), m1 = __ballot_sync(KCNA_FULL, ok[1]);
        int cnt = __popc(m0) + __popc(m1);
        if (!cnt) continue;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(cand_cnt + u, (uint32_t)cnt);
        base = __shfl_sync(KCNA_FULL, base, 0);
        const uint64_t s0 = (uint64_t)u * CB; // whole slots, joiner 0 (no credit)
        if (ok[0]) {
            uint32_t p = base + __popc(m0 & kcna_lanemask_lt());
            if (p < CB) kcna_cand_put(cand, s0 + p, keys[0], 0u);
        }
        if (ok[1]) {
            uint32_t p = base + __popc(m0) + __popc(m1 & kcna_lanemask_lt());
            if (p < CB) kcna_cand_put(cand, s0 + p, keys[1], 0u);
        }
    }
    cc = kcna_warp_sum(cc);
    if (lane == 0 && cc) atomicAdd(s_cc, cc);
    __syncthreads();
}

template <int RMAX>
constexpr size_t p2k_smem_bytes() {
    return (size_t)(RMAX * PJP + PJC * PJP + RMAX * (PJC + 1)) * sizeof(float);
}

// RMAX = 32: nodes with at most 32 pushers (almost all), 22 KB of shared memory
// so eight blocks fit per SM; RMAX = 128: the other nodes, in row tiles of 128.
template <int RMAX, class R>
__global__ void __launch_bounds__(PJT) p2k_join_kernel(R rows, int ld, uint32_t N,
                                                       const uint64_t *__restrict__ off,
                                                       const uint32_t *__restrict__ rnn,
                                                       const uint32_t *__restrict__ g_ids,
                                                       const uint32_t *__restrict__ g_deg,
                                                       const uint8_t *__restrict__ g_isnew, uint32_t W,
                                                       const float *__restrict__ radius, uint64_t *__restrict__ cand,
                                                       uint32_t *__restrict__ cand_cnt, uint32_t CB,
                                                       unsigned long long *comps) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *s_As = reinterpret_cast<float *>(smem); // RMAX x PJP
    float *s_Bs = s_As + RMAX * PJP;               // PJC x PJP
    float *s_D = s_Bs + PJC * PJP;                 // RMAX x (PJC+1)
    __shared__ uint32_t s_u[RMAX], s_w[PJC];
    __shared__ uint8_t s_unew[RMAX], s_wnew[PJC];
    __shared__ unsigned long long s_cc;
    __shared__ int s_n;
    const uint32_t q = blockIdx.x;
    const uint64_t r0 = off[q], r1 = off[q + 1];
    const int deg = (int)min(g_deg[q], W);
    if (r0 == r1 || deg == 0) return;
    if ((RMAX == 32) != (r1 - r0 <= 32)) return; // each node is handled by one of the two instances
    if (threadIdx.x == 0) s_cc = 0;
    for (int c0 = 0; c0 < deg; c0 += PJC) { // graph rows wider than 64: column chunks
        const int nw = min(PJC, deg - c0);
        __syncthreads();
        int wn = 0;
        for (int j = threadIdx.x; j < nw; j += PJT) {
            s_w[j] = g_ids[(uint64_t)q * W + c0 + j];
            s_wnew[j] = g_isnew[(uint64_t)q * W + c0 + j];
            wn |= s_wnew[j];
        }
        // a pair of an old pusher and an old neighbour is skipped
        // (src/kgraph.cpp:2639-2641): without a new neighbour in this chunk only
        // the new pushers enter the tile, and a tile without pushers is skipped
        const bool any_wnew = __syncthreads_or(wn) != 0;
        for (uint64_t t0 = r0; t0 < r1; t0 += RMAX) {
            const int nraw = (int)min((uint64_t)RMAX, r1 - t0);
            __syncthreads();
            if (threadIdx.x == 0) s_n = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < nraw; i += PJT) {
                const uint32_t v = rnn[t0 + i];
                if (!any_wnew && !(v & 0x80000000u)) continue;
                const uint32_t u = v & 0x7FFFFFFFu;
                const int k = atomicAdd(&s_n, 1);
                s_u[k] = u < N ? u : 0;
                s_unew[k] = (v & 0x80000000u) ? 1 : 0;
            }
            __syncthreads();
            const int nu = s_n;
            if (nu == 0) continue;
            if (RMAX == 32 || nu <= 32)
                p2k_tile<1>(rows, ld, N, s_u, s_unew, nu, s_w, s_wnew, nw, radius, cand, cand_cnt, CB, s_As, s_Bs, s_D,
                            &s_cc);
            else if (nu <= 64)
                p2k_tile<RMAX >= 64 ? 2 : 1>(rows, ld, N, s_u, s_unew, nu, s_w, s_wnew, nw, radius, cand, cand_cnt, CB,
                                             s_As, s_Bs, s_D, &s_cc);
            else
                p2k_tile<RMAX >= 128 ? 4 : 1>(rows, ld, N, s_u, s_unew, nu, s_w, s_wnew, nw, radius, cand, cand_cnt, CB,
                                              s_As, s_Bs, s_D, &s_cc);
        }
    }
    if (threadIdx.x == 0 && s_cc) atomicAdd(comps, s_cc);
}

PruneRule make_rule(const kcna_params *p, int kind) {
    PruneRule r;
    r.kind = kind;
    r.t3 = 3.0f * p->tau;
    r.thr = kcna_alpha_threshold(p->angle);
    return r;
}

kcna_status exclusive_scan(kcna_ctx *c, const uint32_t *in, uint64_t n, uint64_t *out, uint64_t *total_h) {
    // out has n+1 entries; out[n] = total
    uint32_t nb = kcna_div_up(std::max<uint64_t>(n, 1), (uint64_t)SCAN_T * SCAN_E);
    uint64_t *sums = nullptr;
    KCNA_TRY(kcna_alloc(c, &sums, nb + 1, "scan sums"));
    scan_block_sums<<<nb, SCAN_T, 0, c->stream>>>(in, n, sums);
    scan_sums_serial<<<1, 1, 0, c->stream>>>(sums, nb, sums + nb);
    scan_apply<<<nb, SCAN_T, 0, c->stream>>>(in, n, sums, out);
    c->launches += 3;
    kcna_status s = kcna_cuda_check(c, cudaMemcpyAsync(out + n, sums + nb, 8, cudaMemcpyDeviceToDevice, c->stream),
                                    "scan total");
    if (s == KCNA_OK && total_h)
        s = kcna_cuda_check(c, cudaMemcpyAsync(total_h, sums + nb, 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "scan sync");
    kcna_release(c, sums);
    return s;
}

} // namespace

kcna_status kcna_exclusive_scan_u32(kcna_ctx *c, const uint32_t *in, uint64_t n, uint64_t *out, uint64_t *total_h) {
    return exclusive_scan(c, in, n, out, total_h);
}

// ---- incremental prune -----------------------------------------------------
// A node's kept list is a function of its first S = max(maxc, 2) pool entries
// (ids and distances; the two flag bits of a key do not enter), of
// min(count, S), of the rows and of the prune's parameters.  Within a build the
// prune runs again after every pool refinement, and many pools come through a
// refinement unchanged (C2 1M: a quarter of the nodes after the first
// BridgeView round, three quarters after the second), so a later prune
// compares every pool prefix with the snapshot of the previous prune, lists
// the nodes whose prefix changed (and takes their new prefix into the
// snapshot), restores the other rows from the graph that prune wrote, and
// prunes the listed nodes only.  Warp per node; 8-byte keys read coalesced.
__global__ void prune_diff_kernel(const uint64_t *__restrict__ pool, const uint32_t *__restrict__ pool_cnt,
                                  uint32_t cap, uint32_t N, uint32_t S, uint64_t *__restrict__ snap,
                                  uint32_t *__restrict__ snap_cnt, uint32_t *__restrict__ list,
                                  uint32_t *__restrict__ list_cnt) {
    const int lane = kcna_lane();
    const uint32_t wpb = blockDim.x >> 5;
    for (uint32_t q = blockIdx.x * wpb + (threadIdx.x >> 5); q < N; q += gridDim.x * wpb) {
        const uint32_t cnt = pool_cnt[q];
        const uint32_t m = min(cnt, S), ms = min(snap_cnt[q], S);
        const uint64_t *pr = pool + (uint64_t)q * cap;
        uint64_t *sr = snap + (uint64_t)q * S;
        uint64_t d = 0;
        for (uint32_t i = lane; i < m; i += 32) d |= (pr[i] ^ sr[i]) & ~(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW);
        if (!__any_sync(KCNA_FULL, d != 0) && m == ms) continue;
        for (uint32_t i = lane; i < m; i += 32) sr[i] = pr[i];
        if (lane == 0) {
            snap_cnt[q] = cnt;
            list[atomicAdd(list_cnt, 1u)] = q;
        }
    }
}

kcna_status kcna_graph_alloc(kcna_ctx *c, uint32_t W) {
    const uint64_t N = c->n;
    if (c->W == W && c->g_ids) return KCNA_OK;
    c->W = W;
    KCNA_TRY(kcna_alloc(c, &c->g_ids, N * W, "graph ids"));
    KCNA_TRY(kcna_alloc(c, &c->g_dist, N * W, "graph dists"));
    KCNA_TRY(kcna_alloc(c, &c->g_isnew, N * W, "graph flags"));
    KCNA_TRY(kcna_alloc(c, &c->g_deg, N, "graph degrees"));
    KCNA_TRY(kcna_alloc(c, &c->g_old, N * W, "previous graph"));
    KCNA_TRY(kcna_alloc(c, &c->g_old_deg, N, "previous degrees"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->g_deg, 0, N * 4, c->stream), "memset"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->g_old_deg, 0, N * 4, c->stream), "memset"));
    if (!c->counters) KCNA_TRY(kcna_alloc(c, &c->counters, 64, "counters"));
    return KCNA_OK;
}

kcna_status kcna_prune_all(kcna_ctx *c, const kcna_params *p, int kind, uint64_t *comps) {
    if (!c->has_pools) return kcna_fail(c, KCNA_E_STATE, "prune: no pools (run NN-descent or set pools first)");
    const uint32_t range = p->nsg_R;
    if (range == 0 || range > 128) return kcna_fail(c, KCNA_E_ARG, "nsg_R must be in [1, 128]");
    KCNA_TRY(kcna_graph_alloc(c, std::max<uint32_t>(c->W, range + 8)));
    PruneRule rule = make_rule(p, kind);
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters + 16, 0, 8, c->stream), "memset"));
    const size_t sm = (size_t)PW * 2 * range * 4;
    const int maxc = (int)std::min(p->search_K, c->cap);
    const bool gram = kcna_prune_tc_ok(c, kind, (int)range, maxc, p->angle);
    const bool fp8 = !gram && kcna_prune_fp8_ok(c, kind, (int)range, maxc);
    // incremental prune (prune_diff_kernel) for the Gram-tile and FP32 prunes
    const char *env = getenv("KCNA_PRUNE_INCREMENTAL");
    const bool inc_on = !fp8 && !(env && env[0] == '0');
    const uint64_t N = c->n, W = c->W;
    const uint32_t S = std::min<uint32_t>(c->cap, (uint32_t)std::max(maxc, 2));
    uint32_t sig[10] = {c->n, c->W, c->cap, S, (uint32_t)kind, range, (uint32_t)maxc,
                        gram ? 2u : c->bf16_exact ? 1u : 0u, 0u, 0u};
    memcpy(&sig[8], &rule.t3, 4);
    memcpy(&sig[9], &p->angle, 4);
    const bool inc = inc_on && c->inc_valid && memcmp(sig, c->inc_sig, sizeof sig) == 0;
    KCNA_TRY(kcna_phase_begin(c));
    uint32_t n_items = c->n;
    const uint32_t *list = nullptr;
    if (!inc) {
        int ds = 0;
        while (ds < 10 && sig[ds] == c->inc_sig[ds]) ++ds;
        kcna_log(c, p, "prune: all %u nodes (%s, parameter word %d)", c->n,
                 !inc_on ? "incremental prune off" : c->inc_valid ? "new parameters" : "first prune", ds);
    }
    c->inc_valid = false; // until this prune's rows are saved
    if (inc) {
        uint32_t *list_cnt = reinterpret_cast<uint32_t *>(c->counters + 52);
        KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(list_cnt, 0, 4, c->stream), "memset"));
        prune_diff_kernel<<<std::max(1, c->num_sms) * 8, 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, c->n, S,
                                                                              c->inc_snap, c->inc_cnt, c->inc_list,
                                                                              list_cnt);
        KCNA_LAUNCHED(c);
        KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "prune_diff_kernel"));
        // the previous prune's rows (the link has rewritten the graph since); the listed nodes are pruned over them
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->g_ids, c->inc_ids, N * W * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->g_dist, c->inc_dist, N * W * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->g_deg, c->inc_deg, N * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&n_items, list_cnt, 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
        KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "prune diff sync"));
        if (n_items > c->n) return kcna_fail(c, KCNA_E_CUDA, "prune: changed-node count out of range");
        c->prune_skipped += c->n - n_items;
        list = c->inc_list;
        kcna_log(c, p, "prune: %u of %u pools changed since the previous prune", n_items, c->n);
    }
    if (gram) { // Gram-exact rows: occlusion masks from tensor-core tiles
        if (list)
            KCNA_TRY(kcna_prune_tc_launch(c, kind, rule.t3, p->angle, (int)range, maxc, c->counters + 16, nullptr, 0,
                                          nullptr, list, n_items, true));
        else
            KCNA_TRY(kcna_prune_tc_launch(c, kind, rule.t3, p->angle, (int)range, maxc, c->counters + 16));
    } else if (fp8) { // float rows, high d: FP8 screen, FP32 where undecided
        uint32_t *resume = nullptr;
        KCNA_TRY(kcna_scratch(c, (size_t)c->n * 4, reinterpret_cast<void **>(&resume)));
        uint32_t *resume_cnt = reinterpret_cast<uint32_t *>(c->counters + 48);
        KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters + 48, 0, 16, c->stream), "memset"));
        KCNA_TRY(kcna_prune_fp8_launch(c, c->pool, c->cap, c->pool_cnt, nullptr, c->n, c->n, rule.t3, (int)range, maxc,
                                       resume, resume_cnt, c->counters + 16, c->counters + 49));
        prune_resume_kernel<<<std::max(1, c->num_sms) * 8, PW * 32, sm, c->stream>>>(
            RowsF32{c->X, (int)c->ld}, c->n, c->pool, c->cap, c->pool_cnt, nullptr, rule, (int)range, maxc, 128,
            resume, resume_cnt, c->g_ids, c->g_dist, c->g_deg, c->W, c->counters + 16);
        KCNA_LAUNCHED(c);
        KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "prune_resume_kernel"));
        unsigned long long ex = 0;
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&ex, c->counters + 49, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
        KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "prune sync"));
        c->prune_exact += ex;
    } else if (n_items > 0) {
        if (c->bf16_exact)
            prune_kernel<<<kcna_div_up(n_items, PW), PW * 32, sm, c->stream>>>(
                RowsB16{c->Xh, (int)c->ld}, c->n, c->pool, c->pool_cnt, c->cap, rule, (int)range, maxc, c->g_ids,
                c->g_dist, c->g_deg, c->W, c->counters + 16, n_items, list);
        else
            prune_kernel<<<kcna_div_up(n_items, PW), PW * 32, sm, c->stream>>>(
                RowsF32{c->X, (int)c->ld}, c->n, c->pool, c->pool_cnt, c->cap, rule, (int)range, maxc, c->g_ids,
                c->g_dist, c->g_deg, c->W, c->counters + 16, n_items, list);
        KCNA_LAUNCHED(c);
        KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "prune_kernel"));
    }
    bool save = inc_on;
    if (save && !inc) { // first prune of the build (or new parameters): a fresh snapshot of every pool prefix
        kcna_status as = kcna_alloc(c, &c->inc_snap, N * S, "prune snapshot");
        if (as == KCNA_OK) as = kcna_alloc(c, &c->inc_cnt, N, "prune snapshot counts");
        if (as == KCNA_OK) as = kcna_alloc(c, &c->inc_ids, N * W, "pruned ids");
        if (as == KCNA_OK) as = kcna_alloc(c, &c->inc_dist, N * W, "pruned dists");
        if (as == KCNA_OK) as = kcna_alloc(c, &c->inc_deg, N, "pruned degrees");
        if (as == KCNA_OK) as = kcna_alloc(c, &c->inc_list, N, "changed nodes");
        if (as == KCNA_E_OOM) { // no room beside the build: every prune of this build prunes every node
            void *bufs[] = {c->inc_snap, c->inc_cnt, c->inc_ids, c->inc_dist, c->inc_deg, c->inc_list};
            for (void *b : bufs) kcna_release(c, b);
            c->inc_snap = nullptr;
            c->inc_cnt = c->inc_ids = c->inc_deg = c->inc_list = nullptr;
            c->inc_dist = nullptr;
            c->err.clear();
            save = false;
            kcna_log(c, p, "prune: no device memory for the incremental prune's snapshot; full prunes");
        } else if (as != KCNA_OK) {
            return as;
        } else {
            KCNA_TRY(kcna_cuda_check(c, cudaMemcpy2DAsync(c->inc_snap, (size_t)S * 8, c->pool, (size_t)c->cap * 8,
                                                          (size_t)S * 8, N, cudaMemcpyDeviceToDevice, c->stream),
                                     "d2d"));
            KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->inc_cnt, c->pool_cnt, N * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        }
    }
    if (save) { // this prune's rows, for the next prune of the build
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->inc_ids, c->g_ids, N * W * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->inc_dist, c->g_dist, N * W * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->inc_deg, c->g_deg, N * 4, cudaMemcpyDeviceToDevice, c->stream), "d2d"));
        memcpy(c->inc_sig, sig, sizeof sig);
        c->inc_valid = true;
    }
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_PRUNE));
    unsigned long long h = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&h, c->counters + 16, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "prune sync"));
    if (comps) *comps = h;
    c->has_graph = true;
    return KCNA_OK;
}

kcna_status kcna_link_all(kcna_ctx *c, const kcna_params *p, int kind, uint64_t *comps) {
    uint64_t pc = 0;
    KCNA_TRY(kcna_prune_all(c, p, kind, &pc));
    const uint64_t N = c->n;
    const uint32_t W = c->W;
    // reverse-edge CSR: in-degree count, scan, fill
    uint32_t *indeg = nullptr, *cursor = nullptr;
    uint64_t *rev = nullptr;
    uint64_t *off = nullptr;
    kcna_status s = KCNA_OK;
    auto cleanup = [&]() {
        kcna_release(c, indeg);
        kcna_release(c, cursor);
        kcna_release(c, rev);
        kcna_release(c, off);
    };
    if ((s = kcna_alloc(c, &indeg, N, "indeg")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &cursor, N, "cursor")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &off, N + 1, "offsets")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_phase_begin(c)) != KCNA_OK) return cleanup(), s;
    cudaMemsetAsync(indeg, 0, N * 4, c->stream);
    cudaMemsetAsync(cursor, 0, N * 4, c->stream);
    rev_count_kernel<<<kcna_div_up(N * W, 256), 256, 0, c->stream>>>(c->g_ids, c->g_deg, (uint32_t)N, W, indeg);
    KCNA_LAUNCHED(c);
    uint64_t E = 0;
    if ((s = exclusive_scan(c, indeg, N, off, &E)) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &rev, std::max<uint64_t>(E, 1), "reverse edges")) != KCNA_OK) return cleanup(), s;
    rev_fill_kernel<<<kcna_div_up(N * W, 256), 256, 0, c->stream>>>(c->g_ids, c->g_dist, c->g_deg, (uint32_t)N, W,
                                                                     off, cursor, rev);
    KCNA_LAUNCHED(c);
    PruneRule rule = make_rule(p, kind);
    cudaMemsetAsync(c->counters + 17, 0, 8, c->stream);
    // warp per node for the common node, the block kernel for the few larger ones
    uint32_t *blist = nullptr, *bcnt = nullptr;
    if ((s = kcna_alloc(c, &blist, N + 1, "link big list")) != KCNA_OK) return cleanup(), s;
    bcnt = blist + N;
    cudaMemsetAsync(bcnt, 0, 4, c->stream);
    // FP8 screen (float rows, high d) or Gram-exact rows: the warp kernel
    // stages its sorted lists for the reversed prune, which a tile prune then
    // takes (lists of at most LW_CAP entries; larger ones stay on the block kernel)
    const bool gram = kcna_prune_tc_ok(c, kind, (int)p->nsg_R, LW_CAP, p->angle);
    const bool fp8 = !gram && kcna_prune_fp8_ok(c, kind, (int)p->nsg_R, 1);
    const bool staged = gram || fp8;
    uint64_t *stage = nullptr;
    uint32_t *stage_meta = nullptr; // nodes, counts, resume list (N each), staged count, resume count
    if (staged) {
        if ((s = kcna_alloc(c, &stage, N * LW_CAP + 2, "link stage")) != KCNA_OK) return cleanup(), s;
        if ((s = kcna_alloc(c, &stage_meta, 3 * N + 2, "link stage lists")) != KCNA_OK) {
            kcna_release(c, stage);
            return cleanup(), s;
        }
        cudaMemsetAsync(stage_meta + 3 * N, 0, 8, c->stream);
    }
    uint32_t *st_nodes = staged ? stage_meta : nullptr, *st_cnt = staged ? stage_meta + N : nullptr;
    uint32_t *st_resume = staged ? stage_meta + 2 * N : nullptr, *st_n = staged ? stage_meta + 3 * N : nullptr;
    auto launch_link = [&](auto rows) -> kcna_status {
        int per_sm = 0;
        KCNA_TRY(kcna_cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, link_warp_kernel<decltype(rows)>,
                                                                                 LW_WARPS * 32, 0),
                                 "link occupancy"));
        const uint32_t grid = (uint32_t)std::min<uint64_t>(kcna_div_up(N, LW_WARPS),
                                                           (uint64_t)std::max(c->num_sms, 1) * std::max(per_sm, 1));
        link_warp_kernel<<<grid, LW_WARPS * 32, 0, c->stream>>>(rows, (uint32_t)N, rule, (int)p->nsg_R, c->g_ids,
                                                                c->g_dist, c->g_deg, W, off, rev, c->counters + 17,
                                                                blist, bcnt, stage, st_nodes, st_cnt, st_n);
        KCNA_LAUNCHED(c);
        uint32_t hb[2] = {0u, 0u};
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&hb[0], bcnt, 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
        if (staged)
            KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&hb[1], st_n, 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
        KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "link sync"));
        if (hb[0] > 0) {
            link_merge_kernel<<<hb[0], LT, 0, c->stream>>>(rows, (uint32_t)N, rule, (int)p->nsg_R, c->g_ids, c->g_dist,
                                                           c->g_deg, W, off, rev, c->counters + 17, c->d_err, blist);
            KCNA_LAUNCHED(c);
        }
        if (gram && hb[1] > 0) // reversed prunes of the staged lists on Gram-exact tiles (no search_K cap)
            KCNA_TRY(kcna_prune_tc_launch(c, kind, rule.t3, p->angle, (int)p->nsg_R, LW_CAP, c->counters + 17, stage,
                                          LW_CAP, st_cnt, st_nodes, hb[1]));
        if (fp8 && hb[1] > 0) { // reversed prunes of the staged lists: FP8 tiles, FP32 where undecided or unfinished
            KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters + 49, 0, 8, c->stream), "memset"));
            KCNA_TRY(kcna_prune_fp8_launch(c, stage, LW_CAP, st_cnt, st_nodes, hb[1], 0xFFFFFFFFu, rule.t3,
                                           (int)p->nsg_R, 0x7FFFFFFF, st_resume, st_n + 1, c->counters + 17,
                                           c->counters + 49));
            prune_resume_kernel<<<std::max(1, c->num_sms) * 8, PW * 32, (size_t)PW * 2 * p->nsg_R * 4, c->stream>>>(
                rows, 0xFFFFFFFFu, stage, LW_CAP, st_cnt, st_nodes, rule, (int)p->nsg_R, 0x7FFFFFFF, 128, st_resume,
                st_n + 1, c->g_ids, c->g_dist, c->g_deg, W, c->counters + 17);
            KCNA_LAUNCHED(c);
            unsigned long long ex = 0;
            KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&ex, c->counters + 49, 8, cudaMemcpyDeviceToHost, c->stream),
                                     "d2h"));
            KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "link sync"));
            c->prune_exact += ex;
        }
        return kcna_cuda_check(c, cudaGetLastError(), "link kernels");
    };
    if (c->bf16_exact)
        s = launch_link(RowsB16{c->Xh, (int)c->ld});
    else
        s = launch_link(RowsF32{c->X, (int)c->ld});
    kcna_release(c, blist);
    if (stage) kcna_release(c, stage);
    if (stage_meta) kcna_release(c, stage_meta);
    unsigned long long h = 0;
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(&h, c->counters + 17, 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK) s = kcna_phase_end(c, KCNA_PHASE_LINK);
    cleanup();
    if (comps) *comps = pc + h;
    return s == KCNA_OK ? kcna_check_device_err(c, "link") : s;
}

kcna_status kcna_search_device(kcna_ctx *c, const float *dQ, uint32_t m, const uint32_t *d_init, uint32_t L,
                               uint32_t k, uint32_t *d_out_ids, float *d_out_d) {
    if (!c->has_graph) return kcna_fail(c, KCNA_E_STATE, "search: no graph");
    if (L == 0 || L > 2048 || k == 0 || k > L) return kcna_fail(c, KCNA_E_ARG, "search: need 0 < k <= L <= 2048");
    const uint32_t vwords = (c->n + 31) / 32;
    uint32_t blocks = std::max<uint32_t>(1, std::min<uint32_t>(kcna_div_up(m, BW), (uint32_t)c->num_sms * 4));
    uint64_t slots = (uint64_t)blocks * BW;
    void *vis = nullptr;
    KCNA_TRY(kcna_scratch2(c, slots * vwords * 4, &vis));
    size_t sm = (size_t)BW * (L + 1) * 8;
    KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(beam_search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)std::max<size_t>(sm, 48 * 1024)),
                             "attr"));
    beam_search_kernel<<<blocks, BW * 32, sm, c->stream>>>(c->X, (int)c->ld, c->n, c->g_ids, c->g_deg, c->W, dQ, m,
                                                           d_init, (int)L, (int)k, (uint32_t *)vis, vwords, d_out_ids,
                                                           d_out_d);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "beam_search");
}

// ComputeEp (src/kgraph.cpp:1528-1536): centroid of all rows, beam search of
// width search_L seeded with the pool of a random node and random fill.
kcna_status kcna_compute_ep(kcna_ctx *c, const kcna_params *p, uint64_t seed) {
    const uint32_t d = c->d, ld = c->ld;
    const uint32_t nrows = c->n_total;
    const uint32_t nb = kcna_div_up(nrows, CB_ROWS);
    double *part = nullptr;
    float *center = nullptr;
    uint32_t *init = nullptr, *oid = nullptr;
    float *od = nullptr;
    kcna_status s = KCNA_OK;
    auto cleanup = [&]() {
        kcna_release(c, part);
        kcna_release(c, center);
        kcna_release(c, init);
        kcna_release(c, oid);
        kcna_release(c, od);
    };
    const uint32_t Lw = std::max<uint32_t>(1, std::min<uint32_t>(p->search_L, c->n - 1));
    if ((s = kcna_alloc(c, &part, (size_t)nb * d, "centroid")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &center, ld, "center")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &init, Lw, "init ids")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &oid, Lw, "ep ids")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &od, Lw, "ep dists")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_phase_begin(c)) != KCNA_OK) return cleanup(), s;
    centroid_partial_kernel<<<nb, 128, 0, c->stream>>>(c->X, (int)ld, nrows, (int)d, part);
    centroid_final_kernel<<<1, 128, 0, c->stream>>>(part, nb, (int)d, (int)ld, nrows, center);
    c->launches += 2;
    // init ids: first search_L pool entries of a random node, then random distinct ids
    std::mt19937 rng((uint32_t)seed);
    uint32_t init_point = rng() % c->n;
    uint32_t cnt = 0;
    std::vector<uint64_t> pk(Lw);
    cudaMemcpyAsync(&cnt, c->pool_cnt + init_point, 4, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(pk.data(), c->pool + (uint64_t)init_point * c->cap, (size_t)std::min(Lw, c->cap) * 8,
                    cudaMemcpyDeviceToHost, c->stream);
    if ((s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "ep d2h")) != KCNA_OK) return cleanup(), s;
    std::vector<uint32_t> ids;
    std::set<uint32_t> seen;
    for (uint32_t i = 0; i < Lw && i < cnt && i < c->cap; ++i) {
        uint32_t id = (uint32_t)(pk[i] & 0xFFFFFFFFull) >> 2;
        if (id < c->n && seen.insert(id).second) ids.push_back(id);
    }
    while (ids.size() < Lw) {
        uint32_t id = rng() % c->n;
        if (seen.insert(id).second) ids.push_back(id);
    }
    cudaMemcpyAsync(init, ids.data(), Lw * 4, cudaMemcpyHostToDevice, c->stream);
    if ((s = kcna_search_device(c, center, 1, init, Lw, 1, oid, od)) != KCNA_OK) return cleanup(), s;
    uint32_t ep = 0;
    cudaMemcpyAsync(&ep, oid, 4, cudaMemcpyDeviceToHost, c->stream);
    s = kcna_phase_end(c, KCNA_PHASE_EP);
    cleanup();
    if (s == KCNA_OK) c->ep = ep < c->n ? ep : 0;
    return s;
}

kcna_status kcna_tree_grow(kcna_ctx *c, const kcna_params *p, uint64_t seed) {
    const uint32_t N = c->n, words = (N + 31) / 32;
    uint32_t *vis = nullptr, *qa = nullptr, *qb = nullptr, *cntd = nullptr, *targeted = nullptr, *localmin = nullptr;
    kcna_status s = KCNA_OK;
    auto cleanup = [&]() {
        kcna_release(c, vis);
        kcna_release(c, qa);
        kcna_release(c, qb);
        kcna_release(c, cntd);
        kcna_release(c, targeted);
        kcna_release(c, localmin);
    };
    if ((s = kcna_alloc(c, &vis, words, "visited")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &qa, N, "frontier")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &qb, N, "frontier")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &cntd, 1, "count")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &targeted, words, "marks")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &localmin, words, "marks")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_phase_begin(c)) != KCNA_OK) return cleanup(), s;
    // BFS levels from the nf nodes in qa (already marked reached)
    auto bfs = [&](uint32_t nf) -> kcna_status {
        for (uint32_t level = 0; nf > 0 && level < N; ++level) {
            cudaMemsetAsync(cntd, 0, 4, c->stream);
            bfs_expand_kernel<<<kcna_div_up((uint64_t)nf * 32, 256), 256, 0, c->stream>>>(c->g_ids, c->g_deg, c->W,
                                                                                          N, qa, nf, vis, qb, cntd);
            KCNA_LAUNCHED(c);
            cudaMemcpyAsync(&nf, cntd, 4, cudaMemcpyDeviceToHost, c->stream);
            KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "bfs"));
            std::swap(qa, qb);
        }
        return KCNA_OK;
    };
    // reached nodes open for a random attach (list in qb): below nsg_R, else below the width
    auto open_list = [&](uint32_t &n_open, uint32_t &open_limit) -> kcna_status {
        n_open = 0;
        for (int lim = 0; lim < 2 && n_open == 0; ++lim) {
            open_limit = lim == 0 ? p->nsg_R : c->W;
            cudaMemsetAsync(cntd, 0, 4, c->stream);
            collect_open_kernel<<<kcna_div_up(N, 256), 256, 0, c->stream>>>(vis, c->g_deg, N, open_limit, c->W, qb,
                                                                             cntd);
            KCNA_LAUNCHED(c);
            cudaMemcpyAsync(&n_open, cntd, 4, cudaMemcpyDeviceToHost, c->stream);
            KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "open list"));
        }
        return KCNA_OK;
    };
    // attaches the unreached nodes marked in `pick`; the attached ones go to qa, their count to nf
    const unsigned wblocks = kcna_div_up((uint64_t)N * 32, 256);
    auto attach = [&](const uint32_t *pick, uint64_t sd, uint32_t n_open, uint32_t open_limit,
                      uint32_t &nf) -> kcna_status {
        cudaMemsetAsync(cntd, 0, 4, c->stream);
        attach_sources_kernel<<<wblocks, 256, 0, c->stream>>>(
            c->X, (int)c->ld, N, c->pool, c->pool_cnt, c->cap, c->g_ids, c->g_dist, c->g_deg, c->W, p->nsg_R, vis,
            pick, qa, cntd, sd, qb, n_open, open_limit, c->d_err, c->counters + 18);
        KCNA_LAUNCHED(c);
        cudaMemcpyAsync(&nf, cntd, 4, cudaMemcpyDeviceToHost, c->stream);
        KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "attach"));
        if (nf > 0) {
            mark_frontier_kernel<<<kcna_div_up(nf, 256), 256, 0, c->stream>>>(qa, nf, vis);
            KCNA_LAUNCHED(c);
        }
        return KCNA_OK;
    };
    cudaMemsetAsync(vis, 0, (size_t)words * 4, c->stream);
    cudaMemsetAsync(c->counters + 18, 0, 16, c->stream);
    const uint32_t ep = c->ep, bit = 1u << (ep & 31), node0 = 1u;
    cudaMemcpyAsync(vis + (ep >> 5), &bit, 4, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(qa, &ep, 4, cudaMemcpyHostToDevice, c->stream);
    if ((s = bfs(1)) != KCNA_OK) return cleanup(), s;
    {   // node 0 first when the entry point does not reach it (attach skips a reached node)
        uint32_t n_open = 0, open_limit = p->nsg_R, nf = 0;
        cudaMemsetAsync(targeted, 0, (size_t)words * 4, c->stream);
        cudaMemcpyAsync(targeted, &node0, 4, cudaMemcpyHostToDevice, c->stream);
        if ((s = open_list(n_open, open_limit)) != KCNA_OK) return cleanup(), s;
        if ((s = attach(targeted, seed ^ 0x9E3779B97F4A7C15ull, n_open, open_limit, nf)) != KCNA_OK)
            return cleanup(), s;
        if ((s = bfs(nf)) != KCNA_OK) return cleanup(), s;
    }
    for (uint32_t round = 0; round < N; ++round) {
        cudaMemsetAsync(targeted, 0, (size_t)words * 4, c->stream);
        cudaMemsetAsync(localmin, 0, (size_t)words * 4, c->stream);
        cudaMemsetAsync(c->counters + 19, 0, 8, c->stream);
        mark_targets_kernel<<<wblocks, 256, 0, c->stream>>>(c->g_ids, c->g_deg, c->W, N, vis, targeted, localmin,
                                                             c->counters + 19);
        KCNA_LAUNCHED(c);
        unsigned long long unreached = 0;
        cudaMemcpyAsync(&unreached, c->counters + 19, 8, cudaMemcpyDeviceToHost, c->stream);
        if ((s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "tree marks")) != KCNA_OK)
            return cleanup(), s;
        if (unreached == 0) break;
        // sources: unreached and not targeted (pick = ~targeted); none left -> local minima
        invert_kernel<<<kcna_div_up(words, 256), 256, 0, c->stream>>>(targeted, words);
        KCNA_LAUNCHED(c);
        uint32_t n_open = 0, open_limit = p->nsg_R, nf = 0;
        if ((s = open_list(n_open, open_limit)) != KCNA_OK) return cleanup(), s;
        for (int pass = 0; pass < 2 && nf == 0; ++pass)
            if ((s = attach(pass == 0 ? targeted : localmin, seed + round * 2 + pass, n_open, open_limit, nf)) !=
                KCNA_OK)
                return cleanup(), s;
        if (nf == 0) {
            s = kcna_fail(c, KCNA_E_CUDA, "tree_grow: no attach point for an unreached node");
            return cleanup(), s;
        }
        if ((s = bfs(nf)) != KCNA_OK) return cleanup(), s;
    }
    s = kcna_cuda_check(c, cudaGetLastError(), "attach");
    if (s == KCNA_OK) s = kcna_phase_end(c, KCNA_PHASE_TREE);
    unsigned long long att = 0;
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaMemcpy(&att, c->counters + 18, 8, cudaMemcpyDeviceToHost), "d2h");
    c->tree_attached += att;
    cleanup();
    return s == KCNA_OK ? kcna_check_device_err(c, "tree_grow") : s;
}

kcna_status kcna_update_nhoods(kcna_ctx *c, int loopcount) {
    update_nhoods_kernel<<<kcna_div_up((uint64_t)c->n * 32, 256), 256, 0, c->stream>>>(
        c->g_ids, c->g_deg, c->g_old, c->g_old_deg, c->g_isnew, c->n, c->W, loopcount == 0 ? 1 : 0);
    KCNA_LAUNCHED(c);
    return kcna_cuda_check(c, cudaGetLastError(), "update_nhoods");
}

// BridgeView (src/kgraph.cpp:2478-2506): rounds of capped pushes and joins;
// when a round pushes fewer than N*massq_S/2 entries the rest is pushed and
// the final join runs.
kcna_status kcna_bridge_view(kcna_ctx *c, const kcna_params *p, uint32_t maxl, int loopcount, uint64_t *comps) {
    const uint32_t N = c->n;
    const uint32_t S_ = std::max<uint32_t>(p->massq_S, 1);
    const int cur_loop = loopcount - 1;
    const uint32_t cur_L = std::min<uint32_t>(p->search_L + (uint32_t)cur_loop * p->step, maxl);
    const uint32_t pre_L = cur_loop > 0 ? std::min<uint32_t>(p->search_L + (uint32_t)(cur_loop - 1) * p->step, maxl) : 0;
    const uint32_t Lp = std::min<uint32_t>(p->search_L + (uint32_t)(loopcount - 1) * p->step, maxl);
    bridge_init_kernel<<<N, 128, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, cur_loop, pre_L, cur_L);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_pools_set_radius(c, maxl));
    uint32_t *tcount = nullptr, *cursor = nullptr, *rnn = nullptr;
    uint64_t *off = nullptr;
    uint64_t rnn_cap = 0;
    uint16_t *nnew = nullptr; // Gram-tile join: new graph neighbours per node (fixed in this call)
    uint8_t *pnew = nullptr;  // and whether a node has a new pusher (per round)
    kcna_status s = KCNA_OK;
    auto cleanup = [&]() {
        kcna_release(c, tcount);
        kcna_release(c, cursor);
        kcna_release(c, rnn);
        kcna_release(c, off);
        kcna_release(c, nnew);
        kcna_release(c, pnew);
    };
    if ((s = kcna_alloc(c, &tcount, N, "push counts")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &cursor, N, "cursor")) != KCNA_OK) return cleanup(), s;
    if ((s = kcna_alloc(c, &off, (uint64_t)N + 1, "offsets")) != KCNA_OK) return cleanup(), s;
    uint64_t total_comps = 0;
    const unsigned wblocks = kcna_div_up((uint64_t)N * 32, 256);
    const bool tc = c->gram_exact && c->W <= 256;
    if (tc) {
        if ((s = kcna_alloc(c, &nnew, N, "new edges")) != KCNA_OK) return cleanup(), s;
        if ((s = kcna_alloc(c, &pnew, N, "new pushers")) != KCNA_OK) return cleanup(), s;
        count_new_edges_kernel<<<wblocks, 256, 0, c->stream>>>(c->g_isnew, c->g_deg, N, c->W, nnew);
        KCNA_LAUNCHED(c);
    }
    if ((s = kcna_cuda_check(c, cudaFuncSetAttribute(p2k_join_kernel<128, RowsF32>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)p2k_smem_bytes<128>()),
                             "p2k smem attr")) != KCNA_OK)
        return cleanup(), s;
    if ((s = kcna_cuda_check(c, cudaFuncSetAttribute(p2k_join_kernel<128, RowsB16>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)p2k_smem_bytes<128>()),
                             "p2k smem attr")) != KCNA_OK)
        return cleanup(), s;
    // the reference loops until a thin round; 100 rounds bound it here
    for (int round = 0; round < 100; ++round) {
        // capped round: count, then the uncapped remainder when the round is thin
        if ((s = kcna_phase_begin(c)) != KCNA_OK) return cleanup(), s;
        cudaMemsetAsync(tcount, 0, (size_t)N * 4, c->stream);
        bridge_update_kernel<<<wblocks, 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, Lp, S_, 1, 0, tcount,
                                                             nullptr, nullptr, nullptr, nullptr);
        KCNA_LAUNCHED(c);
        uint64_t np = 0;
        if ((s = exclusive_scan(c, tcount, N, off, &np)) != KCNA_OK) return cleanup(), s;
        const bool last = (float)np / N / S_ < 0.5f;
        uint64_t np_all = np;
        if (last) { // also count the remainder (pushed after the capped entries are cleared)
            uint32_t *tc2 = nullptr;
            if ((s = kcna_alloc(c, &tc2, N, "push counts")) != KCNA_OK) return cleanup(), s;
            cudaMemsetAsync(tc2, 0, (size_t)N * 4, c->stream);
            // remainder = all flagged in the prefix minus the capped ones: count uncapped, subtract
            bridge_update_kernel<<<wblocks, 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, Lp, S_, 0, 0, tc2,
                                                                 nullptr, nullptr, nullptr, nullptr);
            KCNA_LAUNCHED(c);
            uint64_t np2 = 0;
            s = exclusive_scan(c, tc2, N, off, &np2);
            kcna_release(c, tc2);
            if (s != KCNA_OK) return cleanup(), s;
            np_all = np2; // uncapped count covers the capped pushes too
        }
        // the pushes, grouped by target as they are taken (offsets hold the counts)
        if (!rnn || np_all > rnn_cap) {
            kcna_release(c, rnn);
            rnn = nullptr;
            rnn_cap = std::max<uint64_t>(np_all, (uint64_t)N * S_);
            if ((s = kcna_alloc(c, &rnn, rnn_cap, "rnn")) != KCNA_OK) return cleanup(), s;
        }
        cudaMemsetAsync(cursor, 0, (size_t)N * 4, c->stream);
        if (tc) cudaMemsetAsync(pnew, 0, N, c->stream);
        bridge_update_kernel<<<wblocks, 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, Lp, S_, 1, 1, nullptr,
                                                             off, cursor, rnn, pnew);
        KCNA_LAUNCHED(c);
        if (last) {
            bridge_update_kernel<<<wblocks, 256, 0, c->stream>>>(c->pool, c->pool_cnt, c->cap, N, Lp, S_, 0, 1, nullptr,
                                                                 off, cursor, rnn, pnew);
            KCNA_LAUNCHED(c);
        }
        cudaMemsetAsync(c->counters + 21, 0, 8, c->stream);
        if (tc) {
            if ((s = kcna_p2k_tc_launch(c, off, rnn, nnew, pnew, c->counters + 21)) != KCNA_OK) return cleanup(), s;
        } else if (c->bf16_exact) {
            const RowsB16 rows{c->Xh, (int)c->ld};
            p2k_join_kernel<32><<<N, PJT, p2k_smem_bytes<32>(), c->stream>>>(
                rows, (int)c->ld, N, off, rnn, c->g_ids, c->g_deg, c->g_isnew, c->W, c->radius, c->cand, c->cand_cnt,
                c->CB, c->counters + 21);
            p2k_join_kernel<128><<<N, PJT, p2k_smem_bytes<128>(), c->stream>>>(
                rows, (int)c->ld, N, off, rnn, c->g_ids, c->g_deg, c->g_isnew, c->W, c->radius, c->cand, c->cand_cnt,
                c->CB, c->counters + 21);
        } else {
            const RowsF32 rows{c->X, (int)c->ld};
            p2k_join_kernel<32><<<N, PJT, p2k_smem_bytes<32>(), c->stream>>>(
                rows, (int)c->ld, N, off, rnn, c->g_ids, c->g_deg, c->g_isnew, c->W, c->radius, c->cand, c->cand_cnt,
                c->CB, c->counters + 21);
            p2k_join_kernel<128><<<N, PJT, p2k_smem_bytes<128>(), c->stream>>>(
                rows, (int)c->ld, N, off, rnn, c->g_ids, c->g_deg, c->g_isnew, c->W, c->radius, c->cand, c->cand_cnt,
                c->CB, c->counters + 21);
        }
        if (!tc) c->launches += 2; // the FP32 pair
        unsigned long long h = 0;
        cudaMemcpyAsync(&h, c->counters + 21, 8, cudaMemcpyDeviceToHost, c->stream);
        if ((s = kcna_phase_end(c, KCNA_PHASE_P2K)) != KCNA_OK) return cleanup(), s;
        total_comps += h;
        uint64_t ovf = 0, fl = 0;
        if ((s = kcna_merge(c, maxl, maxl, &ovf, &fl)) != KCNA_OK) return cleanup(), s;
        if (last || round == 99) break;
    }
    cleanup();
    if (comps) *comps = total_comps;
    return kcna_check_device_err(c, "bridge_view");
}
