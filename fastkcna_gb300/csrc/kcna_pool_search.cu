// kcna_pool_search.cu - per-node pool search: each node's own candidate pool
// is the beam of a greedy search over the current graph.
//
// The reference's poolSearch (src/kgraph.cpp:2340-2414), run for every node
// by inSearch (:3667-3688), is the alternative to the P2K BridgeView
// refinement between prune loops (the inSearch calls in the build functions,
// :3761, :3835, :3893, :3950, are commented out there).  For node q with
// cur_L = min(search_L + (loop - 1) step, MAXL):
//   * every pool entry is marked visited and flagged for expansion; on later
//     loops the entries in [pre_L, cur_L) record their previous flag as isnew
//     (:2353-2384);
//   * positions k < cur_L are scanned in order; a flagged entry is expanded:
//     each graph neighbour of its node, unvisited and not q, is marked, its
//     distance to q computed and inserted into q's pool (InsertIntoPool with
//     the pool radius, :1539-1559); the scan restarts at the lowest position
//     an insert landed at (:2386-2410).
// Only q's pool changes, so the result is deterministic.  Where the reference
// reads undefined state the same choices as the oracle are made: the first
// radius is pool[L - 1] for a full pool and +inf otherwise (the reference
// reads the overflow slot, which admits exactly the same inserts into
// pool[0, L)), and positions at or past the pool count are not expanded.
//
// GPU form: persistent, warp per node.  The warp holds the pool (MAXL + 1
// keys) in shared memory, expands one node at a time (its graph row read by
// the lanes, repeated ids resolved to the lowest lane as in sequential order),
// computes each fresh neighbour's canonical distance in its own lane, and
// inserts the fresh neighbours one after another in row order: a count of the
// entries at or below the distance gives the position InsertIntoPool picks
// (including its placement of an equal distance at the end of the pool before
// the last entry), and the tail moves up one slot in 32-entry chunks.  The
// visited set is one byte per base row per warp, stamped with a per-warp
// search counter and cleared every 255 searches; only its own warp touches it,
// and the lanes of a warp test distinct ids, so no atomics are needed.
#include "kcna_internal.h"
#include "kcna_common.cuh"

namespace {

constexpr int PS_WARPS = 8;

struct PoolSearchArgs {
    uint64_t *pool;
    uint32_t *pool_cnt;
    uint32_t cap; // MAXL: a pool holds cap entries, plus the overflow slot in shared memory
    uint32_t N;
    const uint32_t *g_ids;
    const uint32_t *g_deg;
    uint32_t W;
    uint32_t cur_L, pre_L, later_loop;
    uint8_t *visited; // (warps in the grid) x vstride bytes, zero at launch
    uint64_t vstride; // N rounded up to 16
    unsigned long long *comps;
    int *err;
};

__device__ __forceinline__ uint32_t key_dist_bits(uint64_t k) { return (uint32_t)(k >> 32); }

// InsertIntoPool (src/kgraph.cpp:261-298) of (d, id) into the sorted keys
// s[0, L) by the whole warp, with parallel_InsertIntoPool's bookkeeping
// (:1539-1559); returns the position, or cap + 1 when d is beyond the radius.
// The ids are fresh, so the duplicate branch never applies.
__device__ __forceinline__ uint32_t warp_insert(uint64_t *s, uint32_t &L, float &radius, uint32_t cap, float d,
                                                uint32_t id, int lane) {
    if (d > radius) return cap + 1;
    const uint32_t db = __float_as_uint(d);
    uint32_t le = 0; // entries with distance <= d
    for (uint32_t j = lane; j < L; j += 32) le += key_dist_bits(s[j]) <= db ? 1u : 0u;
    le = kcna_warp_sum(le);
    uint32_t pos;
    if (le < L)
        pos = le; // the first entry beyond d (0 when every entry is)
    else
        pos = L == 0 || __uint_as_float(key_dist_bits(s[L - 1])) < d ? L : L - 1;
    for (int base = (int)L - 1; base >= (int)pos; base -= 32) {
        const int j = base - lane;
        uint64_t v = 0;
        if (j >= (int)pos) v = s[j];
        __syncwarp();
        if (j >= (int)pos) s[j + 1] = v;
        __syncwarp();
    }
    if (lane == 0) s[pos] = kcna_key(d, id, (uint32_t)(KCNA_FLAG_NEW | KCNA_FLAG_ISNEW));
    __syncwarp();
    if (L < cap)
        ++L;
    else
        radius = __uint_as_float(key_dist_bits(s[L - 1]));
    return pos;
}

template <class R>
__global__ void __launch_bounds__(PS_WARPS * 32) pool_search_kernel(PoolSearchArgs a, R rows) {
    extern __shared__ __align__(16) uint64_t ps_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t *s = ps_smem + (size_t)warp * (a.cap + 1);
    const uint64_t gw = (uint64_t)blockIdx.x * PS_WARPS + warp, G = (uint64_t)gridDim.x * PS_WARPS;
    uint8_t *vis = a.visited + gw * a.vstride; // 16-byte aligned
    unsigned long long cc = 0;
    uint32_t searches = 0;
    for (uint64_t qq = gw; qq < a.N; qq += G, ++searches) {
        const uint32_t q = (uint32_t)qq;
        if (searches > 0 && searches % 255 == 0) { // stamps 1..255 used up: clear this warp's bytes
            uint4 *v4 = reinterpret_cast<uint4 *>(vis);
            for (uint64_t j = lane; j < a.vstride / 16; j += 32) v4[j] = make_uint4(0, 0, 0, 0);
            __syncwarp();
        }
        const uint8_t stamp = (uint8_t)(searches % 255 + 1);
        uint32_t L = min(a.pool_cnt[q], a.cap);
        const uint64_t *pq = a.pool + (uint64_t)q * a.cap;
        for (uint32_t t = lane; t < L; t += 32) {
            const uint64_t k = pq[t];
            const uint32_t f = (uint32_t)(k & KCNA_FLAG_NEW);
            const bool isnew = a.later_loop && t >= a.pre_L && t < a.cur_L && f;
            s[t] = (k & ~3ull) | KCNA_FLAG_NEW | (isnew ? KCNA_FLAG_ISNEW : 0ull);
            const uint32_t id = kcna_key_id(k);
            if (id < a.N) vis[id] = stamp;
        }
        __syncwarp();
        float radius = L >= a.cap && L > 0 ? __uint_as_float(key_dist_bits(s[L - 1])) : __int_as_float(0x7f800000);
        uint32_t k = 0;
        while (k < a.cur_L) {
            uint32_t nk = a.cur_L;
            if (k < L && (s[k] & KCNA_FLAG_NEW)) {
                const uint64_t e = s[k];
                __syncwarp();
                if (lane == 0) s[k] = e & ~(uint64_t)KCNA_FLAG_NEW;
                __syncwarp();
                const uint32_t n = kcna_key_id(e);
                const uint32_t deg = n < a.N ? min(a.g_deg[n], a.W) : 0u;
                const uint32_t *row = a.g_ids + (uint64_t)n * a.W;
                for (uint32_t m0 = 0; m0 < deg; m0 += 32) {
                    const uint32_t m = m0 + lane;
                    const uint32_t id = m < deg ? row[m] : 0xFFFFFFFFu;
                    const bool cand = m < deg && id < a.N && id != q;
                    // a repeated id within the chunk: only its first lane (row order) tests it
                    const unsigned same = __match_any_sync(KCNA_FULL, cand ? id : 0xFFFFFFFFu);
                    bool fresh = false;
                    if (cand && (__ffs(same) - 1) == lane && vis[id] != stamp) {
                        vis[id] = stamp;
                        fresh = true;
                    }
                    unsigned fm = __ballot_sync(KCNA_FULL, fresh);
                    if (lane == 0) cc += __popc(fm);
                    const float d = fresh ? rows_l2(rows, q, id) : 0.f;
                    while (fm) {
                        const int t = __ffs(fm) - 1;
                        fm &= fm - 1;
                        const float dt = __shfl_sync(KCNA_FULL, d, t);
                        const uint32_t it = __shfl_sync(KCNA_FULL, id, t);
                        const uint32_t r = warp_insert(s, L, radius, a.cap, dt, it, lane);
                        nk = min(nk, r);
                    }
                }
            }
            k = nk <= k ? nk : k + 1;
        }
        uint64_t *pw = a.pool + (uint64_t)q * a.cap;
        for (uint32_t t = lane; t < L; t += 32) pw[t] = s[t];
        if (lane == 0) a.pool_cnt[q] = L;
        __syncwarp();
    }
    cc = kcna_warp_sum(cc);
    if (lane == 0 && cc) atomicAdd(a.comps, cc);
}

} // namespace

kcna_status kcna_pool_search_run(kcna_ctx *c, const kcna_params *p, uint32_t maxl, int loopcount, uint64_t *comps) {
    if (!c->has_pools || !c->has_graph) return kcna_fail(c, KCNA_E_STATE, "pool search: needs pools and a graph");
    if (loopcount < 1) return kcna_fail(c, KCNA_E_ARG, "pool search: loop count starts at 1");
    if (maxl != c->cap) return kcna_fail(c, KCNA_E_STATE, "pool search: pools must hold MAXL entries");
    const uint32_t cur_loop = (uint32_t)loopcount - 1;
    PoolSearchArgs a;
    a.pool = c->pool;
    a.pool_cnt = c->pool_cnt;
    a.cap = c->cap;
    a.N = c->n;
    a.g_ids = c->g_ids;
    a.g_deg = c->g_deg;
    a.W = c->W;
    a.cur_L = (uint32_t)std::min<uint64_t>((uint64_t)p->search_L + (uint64_t)cur_loop * p->step, maxl);
    a.pre_L = cur_loop == 0 ? 0u
                            : (uint32_t)std::min<uint64_t>((uint64_t)p->search_L + (uint64_t)(cur_loop - 1) * p->step, maxl);
    a.later_loop = cur_loop > 0 ? 1u : 0u;
    a.err = c->d_err;
    const size_t sm = (size_t)PS_WARPS * (c->cap + 1) * 8;
    if (sm > 200 * 1024) return kcna_fail(c, KCNA_E_ARG, "pool search: MAXL too large for shared memory");
    auto launch = [&](auto rows) -> kcna_status {
        auto kern = pool_search_kernel<decltype(rows)>;
        KCNA_TRY(kcna_cuda_check(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)std::max<size_t>(sm, 48 * 1024)),
                                 "pool search smem attr"));
        int per_sm = 0;
        KCNA_TRY(kcna_cuda_check(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PS_WARPS * 32, sm),
                                 "pool search occupancy"));
        // visited bytes: one per base row per warp, at most 4 GiB
        uint64_t blocks = (uint64_t)std::max(c->num_sms, 1) * (uint64_t)std::max(per_sm, 1);
        blocks = std::min<uint64_t>(blocks, std::max<uint64_t>(1, (4ull << 30) / (((uint64_t)c->n + 15) * PS_WARPS)));
        blocks = std::min<uint64_t>(blocks, kcna_div_up(c->n, PS_WARPS));
        const uint64_t vstride = ((uint64_t)c->n + 15) & ~15ull;
        const uint64_t vbytes = blocks * PS_WARPS * vstride;
        uint8_t *vis = nullptr;
        KCNA_TRY(kcna_alloc(c, &vis, vbytes, "pool search visited bytes"));
        kcna_status s = kcna_cuda_check(c, cudaMemsetAsync(vis, 0, vbytes, c->stream), "memset");
        if (s == KCNA_OK) s = kcna_cuda_check(c, cudaMemsetAsync(c->counters + 24, 0, 8, c->stream), "memset");
        if (s == KCNA_OK) {
            a.visited = vis;
            a.vstride = vstride;
            a.comps = c->counters + 24;
            kern<<<(unsigned)blocks, PS_WARPS * 32, sm, c->stream>>>(a, rows);
            KCNA_LAUNCHED(c);
            s = kcna_cuda_check(c, cudaGetLastError(), "pool_search_kernel");
        }
        unsigned long long h = 0;
        if (s == KCNA_OK)
            s = kcna_cuda_check(c, cudaMemcpyAsync(&h, c->counters + 24, 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
        if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "pool search sync");
        kcna_release(c, vis);
        if (s == KCNA_OK && comps) *comps = h;
        return s;
    };
    KCNA_TRY(kcna_phase_begin(c));
    if (c->bf16_exact)
        KCNA_TRY(launch(RowsB16{c->Xh, (int)c->ld}));
    else
        KCNA_TRY(launch(RowsF32{c->X, (int)c->ld}));
    KCNA_TRY(kcna_phase_end(c, KCNA_PHASE_P2K));
    return kcna_pools_set_radius(c, maxl);
}
