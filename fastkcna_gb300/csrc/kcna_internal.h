// kcna_internal.h - host-side context of the GB300 FastKCNA build library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kcna.h"

#define KCNA_EMPTY_KEY_H 0xFFFFFFFFFFFFFFFFull
#define KCNA_MAX_ID ((1u << 30) - 1) // ids live in 30 bits of a pool key

struct kcna_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // background file writer (kcna_write_nsg_async): one write in flight; its
    // outcome is read after join
    std::thread writer;
    kcna_status writer_status = KCNA_OK;
    std::string writer_err;
    uint64_t launches = 0;
    int *d_err = nullptr; // device error word (kcna_common.cuh KCNA_DERR_*)

    // rows: n_total x ld floats, ld = d rounded up to 4, padding zero
    float *X = nullptr;
    uint32_t n_total = 0, n = 0, d = 0, ld = 0;
    // BF16 copy of the rows (n_total x ld), present only during a BF16-mode build
    // of data whose every value is exactly representable in BF16
    uint16_t *Xh = nullptr;
    // Gram-exact BF16 mode: the rows are integers and every squared norm is
    // below 2^23 (2^22 when a value is negative), so |x|^2 + |y|^2 - 2<x,y>
    // evaluated by the tensor cores in FP32 equals the canonical FMA-chain
    // distance bit for bit; the local join, the P2K join and the prune then
    // run on tcgen05 Gram tiles.  norms[i] = |x_i|^2 (n_total floats).
    bool gram_exact = false;
    float *norms = nullptr;
    // bf16_exact: Xh holds the rows' values exactly (kernels may read it in
    // place of X).  bf16_screen: the rows are not exact in BF16; Xh holds them
    // rounded to nearest and norms their squared norms, and the local join
    // screens pairs on Gram tiles of the rounded rows with a bound on the
    // rounding error, then recomputes every emitted pair in FP32 (rescore).
    bool bf16_exact = false, bf16_screen = false;
    // fp8_screen (BF16 mode, rows inexact in BF16, d >= 256): the tau-MNG
    // prune screens pairs on FP8 E4M3 Gram tiles (kcna_prune_fp8.cu).  Xq holds
    // the codes (n_total x ldq bytes, ldq = d rounded up to 128, zero padded),
    // qmeta per row {scale, squared norm of the decoded row, bound on the
    // encoding error, 0}.
    bool fp8_screen = false;
    uint8_t *Xq = nullptr;
    float4 *qmeta = nullptr;
    uint32_t ldq = 0;

    // candidate pools: n x cap keys (kcna_common.cuh), counts, filter radius
    uint32_t cap = 0;
    uint64_t *pool = nullptr;
    uint32_t *pool_cnt = nullptr;
    float *radius = nullptr;

    // NN-descent state
    uint32_t S = 0, Rr = 0, RB = 0, CB = 0, fwd_new_cap = 0, fwd_old_cap = 0;
    uint32_t *M = nullptr;
    float *radiusM = nullptr;
    uint8_t *found = nullptr;
    uint32_t *fwd_new = nullptr, *fwd_new_cnt = nullptr;
    uint32_t *fwd_old = nullptr, *fwd_old_cnt = nullptr;
    uint32_t *rnew = nullptr, *rnew_cnt = nullptr;
    uint32_t *rold = nullptr, *rold_cnt = nullptr;
    uint64_t *cand = nullptr;
    uint32_t *cand_cnt = nullptr;
    uint32_t *big_list = nullptr, *big_cnt = nullptr; // merge queue of nodes with many candidates
    uint32_t merge_big_last = 0;                      // nodes the previous merge queued
    unsigned long long *counters = nullptr; // device scratch counters (64 slots)

    // graph: n x W ids / dists / isnew flags, degrees; previous-loop ids
    uint32_t W = 0;
    uint32_t *g_ids = nullptr, *g_deg = nullptr, *g_old = nullptr, *g_old_deg = nullptr;
    float *g_dist = nullptr;
    uint8_t *g_isnew = nullptr;
    uint32_t ep = 0, width = 0;
    bool has_graph = false, has_pools = false;

    // incremental prune (kcna_prune_all): the first S = min(cap, max(maxc, 2))
    // keys and the count of every pool at the previous prune (inc_snap, n x S;
    // inc_cnt), the graph rows that prune wrote (inc_ids / inc_dist, n x W;
    // inc_deg), room for a list of n nodes, and what the kept lists depended on
    // besides the pools (inc_sig).  Dropped with the pools (free_state: every
    // build, upload and set_size), so a build never reuses an earlier build's.
    uint64_t *inc_snap = nullptr;
    uint32_t *inc_cnt = nullptr, *inc_ids = nullptr, *inc_deg = nullptr, *inc_list = nullptr;
    float *inc_dist = nullptr;
    bool inc_valid = false;
    uint32_t inc_sig[10] = {};
    uint64_t prune_skipped = 0; // nodes whose prune the snapshot showed unchanged

    // controls (exact MAXL-NN of sampled nodes) for the recall estimate
    std::vector<uint32_t> control_ids;
    std::vector<uint32_t> control_cache; // the reference's control order for control_cache_n rows
    uint32_t control_cache_n = 0;
    uint32_t *d_controls = nullptr, *d_control_knn = nullptr;
    uint32_t control_k = 0;

    // generic scratch reused by phases
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    void *scratch2 = nullptr;
    size_t scratch2_bytes = 0;

    // device memory cache: blocks from kcna_dev_malloc that kcna_release handed
    // back, kept (by size) for the next kcna_alloc instead of cudaFree, so that
    // repeated builds of one size allocate once; freed at kcna_destroy, or
    // when cudaMalloc runs out of memory
    std::multimap<size_t, void *> free_blocks;
    std::unordered_map<void *, size_t> block_bytes;

    kcna_stats *stats = nullptr;
    double t0 = 0;

    // the learned seed's subsample NN-descent runs in this context, kept
    // across builds so that its buffers stay in its memory cache
    kcna_ctx *seed_sub = nullptr;

    // phase timing with CUDA events on `stream`
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double phase_ms[KCNA_NUM_PHASES] = {};
    uint64_t phase_launches[KCNA_NUM_PHASES] = {};
    uint64_t launches_at_begin = 0;
    uint64_t join_rows = 0, cand_emitted = 0, cand_merged = 0, pool_entries_merged = 0, tree_attached = 0;
    uint64_t prune_exact = 0; // undecided pairs of the FP8-screened prunes recomputed in FP32
};

// Brackets one phase with events on the context stream; end() waits for the
// phase and adds its device time and launch count.
kcna_status kcna_phase_begin(kcna_ctx *c);
kcna_status kcna_phase_end(kcna_ctx *c, int phase);

// error plumbing
kcna_status kcna_fail(kcna_ctx *c, kcna_status s, const std::string &msg);
kcna_status kcna_cuda_check(kcna_ctx *c, cudaError_t e, const char *what);
kcna_status kcna_check_device_err(kcna_ctx *c, const char *phase);
kcna_status kcna_scratch(kcna_ctx *c, size_t bytes, void **out);
kcna_status kcna_scratch2(kcna_ctx *c, size_t bytes, void **out);
#define KCNA_TRY_ALLOC(x)                            \
    do {                                             \
        kcna_status _s = (x);                        \
        if (_s != KCNA_OK) return _s;                \
    } while (0)
// Device memory through the context's cache (kcna_internal.h kcna_ctx::free_blocks).
// All of a context's kernels run on its one stream, so a block released and
// handed out again is ordered after every use of its previous owner.
kcna_status kcna_dev_malloc(kcna_ctx *c, size_t bytes, void **out, const char *what);
void kcna_release(kcna_ctx *c, void *p); // back to the cache; cudaFree for a block not from the cache
void kcna_release_all(kcna_ctx *c);      // cudaFree of every cached block
template <typename T>
kcna_status kcna_alloc(kcna_ctx *c, T **p, size_t count, const char *what) {
    if (*p) {
        kcna_release(c, *p);
        *p = nullptr;
    }
    if (count == 0) return KCNA_OK;
    void *q = nullptr;
    KCNA_TRY_ALLOC(kcna_dev_malloc(c, count * sizeof(T), &q, what));
    *p = static_cast<T *>(q);
    return KCNA_OK;
}
#define KCNA_TRY(x)                                  \
    do {                                             \
        kcna_status _s = (x);                        \
        if (_s != KCNA_OK) return _s;                \
    } while (0)
#define KCNA_LAUNCHED(c) ((c)->launches++)
double kcna_now();
void kcna_log(kcna_ctx *c, const kcna_params *p, const char *fmt, ...);

// kcna_knn.cu: exact k-NN of m query rows (device, m x ld) against rows
// [0, n) of X; q_self (device, may be null) gives a row id to exclude per query.
kcna_status kcna_knn_device(kcna_ctx *c, const float *dQ, uint32_t m, const uint32_t *q_self, uint32_t k,
                            uint32_t *d_out_ids, float *d_out_d);
// gathers rows ids[0..m) of X into dst (m x ld)
kcna_status kcna_gather_rows(kcna_ctx *c, const uint32_t *d_ids, uint32_t m, float *dst);

// kcna_tc.cu: BF16 tensor-core GEMM, C = A * B^T (+ beta * C)
kcna_status kcna_tc_gemm(cudaStream_t s, const void *A, int64_t lda, int a_fp32, int a_trans, const void *B,
                         int64_t ldb, int b_fp32, int b_trans, float *C, int64_t ldc, int M, int N, int K, float beta,
                         int *err);

// kcna_nnd.cu: NN-descent phases
kcna_status kcna_nnd_alloc(kcna_ctx *c, const kcna_params *p, uint32_t maxl);
kcna_status kcna_nnd_init(kcna_ctx *c, const kcna_params *p);
// candidate buffers for a refinement run outside a build (kcna_refine_pools), when absent
kcna_status kcna_cand_alloc(kcna_ctx *c, const kcna_params *p);
kcna_status kcna_nnd_join(kcna_ctx *c, const kcna_params *p, int iter, uint64_t *n_comps);  // iter 0: init lists
// Merges every node's candidate buffer into its pool.  credit_found: the
// candidates of an NN-descent join, whose joiners (stored beside their keys) are credited with
// found flags for the entries they inserted below K.
kcna_status kcna_merge(kcna_ctx *c, uint32_t limit, uint32_t K, uint64_t *overflow, uint64_t *flagged_topk,
                       uint64_t *merged = nullptr, uint64_t *inserted = nullptr, bool credit_found = false);
// cos(angle) as the reference's alpha-PG prune computes it (src/kgraph.cpp:3160-3161:
// the float angle / 180 times the double pi, cos in double, stored as float).
inline float kcna_alpha_threshold(float angle) {
    return (float)std::cos((double)(angle / 180.0f) * 3.14159265358979323846264);
}
// Occlusion prune on tcgen05 Gram tiles (kcna_prune_tc.cu); requires c->gram_exact.
// alpha-PG takes it for angles up to 60 degrees only (angle: degrees).
bool kcna_prune_tc_ok(const kcna_ctx *c, int kind, int range, int maxc, float angle);
// Node mode (nodes null): each node's pool.  List mode: n_items staged
// candidate lists (pool-format keys, `stride` apart, cnt[k] each) of nodes[k].
// Pool-list mode (pool_list; keys, stride and cnt unused): the pools of the
// n_items nodes nodes[k].
kcna_status kcna_prune_tc_launch(kcna_ctx *c, int kind, float t3, float angle, int range, int maxc,
                                 unsigned long long *comps, const uint64_t *keys = nullptr, uint64_t stride = 0,
                                 const uint32_t *cnt = nullptr, const uint32_t *nodes = nullptr,
                                 uint32_t n_items = 0, bool pool_list = false);
// tau-MNG prune of float rows on FP8 E4M3 Gram tiles (kcna_prune_fp8.cu);
// requires c->fp8_screen.  The first 128 candidates of every item are pruned
// on the tiles; items whose scan ran out of them with fewer than range kept
// and more candidates left are appended to `resume` (item indices) for the
// FP32 prune to finish.  keys: candidate keys, row = node (nodes null) or list
// position, `stride` apart, cnt[row] of them.
bool kcna_prune_fp8_ok(const kcna_ctx *c, int kind, int range, int maxc);
kcna_status kcna_fp8_rows(kcna_ctx *c);
kcna_status kcna_prune_fp8_launch(kcna_ctx *c, const uint64_t *keys, uint64_t stride, const uint32_t *cnt,
                                  const uint32_t *nodes, uint32_t n_items, uint32_t n_oracle, float t3, int range,
                                  int maxc, uint32_t *resume, uint32_t *resume_cnt, unsigned long long *comps,
                                  unsigned long long *exact);
// P2K join on tcgen05 Gram tiles (kcna_p2k_tc.cu); requires c->gram_exact.
// nnew[q]: q's graph neighbours flagged new; pnew[q]: 1 when a pusher of q this round is new.
kcna_status kcna_p2k_tc_launch(kcna_ctx *c, const uint64_t *off, const uint32_t *rnn, const uint16_t *nnew,
                               const uint8_t *pnew, unsigned long long *comps);
kcna_status kcna_nnd_sample(kcna_ctx *c, const kcna_params *p, int iter);
kcna_status kcna_controls_setup(kcna_ctx *c, const kcna_params *p, uint32_t maxl);
kcna_status kcna_control_recall(kcna_ctx *c, uint32_t K, float *recall);
kcna_status kcna_pools_set_radius(kcna_ctx *c, uint32_t limit);
kcna_status kcna_nndescent_run(kcna_ctx *c, const kcna_params *p, kcna_stats *st);

// kcna_seed.cu: learned seeding
kcna_status kcna_seed_learned(kcna_ctx *c, const kcna_params *p, kcna_stats *st);
kcna_status kcna_seed_finish(kcna_ctx *c, const kcna_params *p);

// kcna_graph.cu: prune / link / entry point / connectivity / P2K / search
kcna_status kcna_exclusive_scan_u32(kcna_ctx *c, const uint32_t *in, uint64_t n, uint64_t *out, uint64_t *total_h);
kcna_status kcna_graph_alloc(kcna_ctx *c, uint32_t W);
// Drops every state and allocates (zero-padded) device rows for n x d floats.
kcna_status kcna_rows_reset(kcna_ctx *c, uint32_t n, uint32_t d);
kcna_status kcna_prune_all(kcna_ctx *c, const kcna_params *p, int kind, uint64_t *comps);
// CAGRA-style rank prune of the pools into the graph (kcna_cagra.cu).
kcna_status kcna_cagra_prune(kcna_ctx *c, const kcna_params *p);
kcna_status kcna_link_all(kcna_ctx *c, const kcna_params *p, int kind, uint64_t *comps);
kcna_status kcna_compute_ep(kcna_ctx *c, const kcna_params *p, uint64_t seed);
kcna_status kcna_tree_grow(kcna_ctx *c, const kcna_params *p, uint64_t seed);
kcna_status kcna_update_nhoods(kcna_ctx *c, int loopcount);
kcna_status kcna_bridge_view(kcna_ctx *c, const kcna_params *p, uint32_t maxl, int loopcount, uint64_t *comps);
// Per-node pool search over the graph (inSearch; kcna_pool_search.cu).
kcna_status kcna_pool_search_run(kcna_ctx *c, const kcna_params *p, uint32_t maxl, int loopcount, uint64_t *comps);
kcna_status kcna_search_device(kcna_ctx *c, const float *dQ, uint32_t m, const uint32_t *d_init, uint32_t L,
                               uint32_t k, uint32_t *d_out_ids, float *d_out_d);
