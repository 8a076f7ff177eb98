/*
 * kcna.h - C ABI of the GB300 (sm_103a) FastKCNA graph-construction library.
 *
 * This is the drop-in boundary for FastKCNA's build path.  The reference
 * exposes a C++ virtual interface (kgraph::KGraph in src/kgraph.h:113-304)
 * whose data enters through the IndexOracle plugin (src/kgraph.h:63-81) over a
 * caller-owned Matrix<float> (src/kgraph-data.h:97-288).  Every entry point
 * below is plain C: pointers, sizes and status codes, no C++ or torch types, so
 * that a C++ facade (kgraph_gb300.h), a ctypes stub or any other FFI can bind
 * it.  Each function names the reference interface it replaces.
 *
 * Threading: one context per host thread.  A context owns one CUDA stream on
 * one device and all device memory of one build.
 * Errors: every call returns kcna_status; kcna_last_error() gives the text.
 */
#ifndef KCNA_H
#define KCNA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    KCNA_OK = 0,
    KCNA_E_ARG = 1,     /* maps to kgraph::invalid_argument (src/kgraph.h:363-366) */
    KCNA_E_OOM = 2,     /* device or host allocation failed */
    KCNA_E_CUDA = 3,    /* a CUDA call failed; maps to kgraph::runtime_error */
    KCNA_E_TIMEOUT = 4, /* a bounded device-side wait gave up (error flag set) */
    KCNA_E_IO = 5,      /* maps to kgraph::io_error (src/kgraph.h:373-376) */
    KCNA_E_STATE = 6,   /* call order violated (e.g. prune before build) */
    KCNA_E_LIMIT = 7    /* a data-dependent capacity was exceeded: more than 1024 rows
                           tie at the k-th distance of an exact k-NN query */
} kcna_status;

/* Graph kinds.  The numbers equal the reference's PG_type column of the run CSV
 * (src/kgraph.cpp:3757 HNSW=2, :3816 NSG=1, :3874 TauMNG=3, :3931 AlphaPG=4). */
typedef enum {
    KCNA_NSG = 1,
    KCNA_HNSW_LAYER = 2, /* NSG-style layer without tree_grow (buildHNSWLayer, :2326-2337) */
    KCNA_TAUMNG = 3,
    KCNA_ALPHAPG = 4,
    KCNA_CAGRA = 5 /* kcna_prune only: CAGRA-style rank prune (BuildCagra, :2818-2829) */
} kcna_kind;

/* Refinement of the pools between prune loops (kcna_params.refine). */
typedef enum {
    KCNA_REFINE_BRIDGE_VIEW = 0, /* P2K BridgeView (src/kgraph.cpp:2478-2663), the reference's builds */
    KCNA_REFINE_POOL_SEARCH = 1  /* per-node pool search, inSearch (:2340-2414, :3667-3688) */
} kcna_refine;

/* Distance screening forms for the local join, the P2K join and the prune. */
typedef enum {
    KCNA_SCREEN_FP32 = 0, /* plain FP32, the drop-in */
    KCNA_SCREEN_BF16 = 1  /* BF16 tensor-core Gram screen + FP32 re-rank of survivors (d <= 128);
                             at d >= 256 the tau-MNG prune screens on FP8 E4M3 Gram tiles with
                             per-vector scales and recomputes undecided pairs in FP32 */
} kcna_screen;

/* Build parameters.  Field meaning and defaults follow kgraph::KGraph::IndexParams
 * (src/kgraph.h:116-170, defaults :12-40) and the CLI flags (src/fastnsg.cpp:53-94). */
typedef struct {
    uint32_t K;          /* -K, default 25 */
    uint32_t L;          /* -L, default 100 */
    uint32_t S;          /* -S, default 10 */
    uint32_t R;          /* -R, default 100 */
    uint32_t iterations; /* -I, default 30 */
    uint32_t controls;   /* --controls, default 100 */
    uint32_t seed;       /* --seed, default 2024 */
    uint32_t nthreads;   /* --nthreads (host threads of CPU helpers) */
    float delta;         /* --delta, default 0.002 */
    float recall;        /* --recall, default 0.95 */
    uint32_t nsg_R;      /* --nsg_R, default 50 */
    uint32_t search_L;   /* --search_L, default 40 */
    uint32_t search_K;   /* --search_K, default 500 */
    uint32_t step;       /* --step, default 10 */
    uint32_t massq_S;    /* --massq_S, default 10 */
    uint32_t loop_i;     /* --loop_i, default 2 */
    float tau;           /* --tau, default 0 */
    float angle;         /* --angle (degrees), default 60 */
    /* GB300 extensions (no counterpart in the reference) */
    uint32_t screen;     /* kcna_screen */
    uint32_t learned_seed; /* 1: seed NN-descent from learned codes (kcna_seed_learned) */
    uint32_t verbosity;  /* 0 silent, 1 per-phase lines on stderr */
    uint32_t refine;     /* kcna_refine: the refinement between prune loops */
    uint32_t reserved[4];
} kcna_params;

/* Fills p with the reference defaults (src/kgraph.h:12-40). */
void kcna_params_default(kcna_params *p);

/* Statistics of one build.  Key names follow the reference's run CSV
 * (SaveResult, src/kgraph.cpp:1725-1807) and IndexInfo (src/kgraph.h:186-198). */
#define KCNA_MAX_ITERS 64
#define KCNA_MAX_LOOPS 16
#define KCNA_NUM_PHASES 12
enum {
    KCNA_PHASE_JOIN = 0,     /* NN-descent local join */
    KCNA_PHASE_MERGE = 1,    /* candidate merge into pools (NN-descent and P2K) */
    KCNA_PHASE_SAMPLE = 2,   /* new/old sampling and reverse lists */
    KCNA_PHASE_PRUNE = 3,    /* occlusion prune of the pools */
    KCNA_PHASE_LINK = 4,     /* reverse edges + re-prune */
    KCNA_PHASE_P2K = 5,      /* P2K pushes and join */
    KCNA_PHASE_EP = 6,       /* centroid + entry-point beam search */
    KCNA_PHASE_TREE = 7,     /* reachability + attach */
    KCNA_PHASE_CONTROLS = 8, /* exact k-NN of the controls + recall */
    KCNA_PHASE_INIT = 9,     /* pool initialisation */
    KCNA_PHASE_OTHER = 10
};
typedef struct {
    uint32_t iterations;       /* NN-descent iterations run */
    uint32_t stop_condition;   /* 0 ITERATION, 1 DELTA, 2 RECALL (IndexInfo::StopCondition) */
    uint32_t maxl;             /* candidate pool size MAXL = max(L,K,search_L,search_K) */
    uint32_t loops;            /* prune/P2K loops run (loop_i+1) */
    float iter_recall[KCNA_MAX_ITERS]; /* control recall@K after each join */
    float iter_delta[KCNA_MAX_ITERS];
    double iter_time[KCNA_MAX_ITERS];  /* seconds since build start ("kgraph time") */
    uint64_t iter_cand_overflow[KCNA_MAX_ITERS]; /* candidates dropped by full buffers */
    float loop_recall[KCNA_MAX_LOOPS + 1]; /* evaluate(): control recall@MAXL, [0] after NN-descent */
    double prune_time[KCNA_MAX_LOOPS];
    double inter_time[KCNA_MAX_LOOPS];
    double tree_grow_time[KCNA_MAX_LOOPS];
    double buildnsg_time[KCNA_MAX_LOOPS];
    double search_time[KCNA_MAX_LOOPS];   /* P2K (BridgeView) seconds per loop */
    double con_time[KCNA_MAX_LOOPS];      /* seconds since start after each loop */
    double nndescent_time;
    double total_time;
    uint64_t n_comps;          /* NN-descent join distance evaluations (kgraph.cpp:1116) */
    uint64_t prune_comps;      /* prune distance evaluations */
    uint64_t bridge_comps;     /* P2K join distance evaluations */
    uint64_t screened_pairs;   /* pairs screened in BF16 (0 in FP32 mode) */
    uint64_t rescored_pairs;   /* screened pairs recomputed in FP32 */
    uint32_t ep;               /* entry point */
    uint32_t width;            /* max out-degree */
    uint32_t aod;              /* average out-degree (CalculateNSG, :2273-2293) */
    uint32_t min_degree, max_degree;
    uint32_t rev_overflow;     /* reverse-list entries dropped because a list was full (RB) */
    uint32_t reserved[2];
    /* Device time per phase, measured with CUDA events on the context stream
     * (milliseconds, summed over the build), and kernel launches per phase.
     * Phases: see KCNA_PHASE_* below. */
    double phase_ms[KCNA_NUM_PHASES];
    uint64_t phase_launches[KCNA_NUM_PHASES];
    uint64_t join_rows;        /* rows gathered by the NN-descent joins (new + old lists) */
    uint64_t cand_emitted;     /* candidates written to buffers (join + P2K) */
    uint64_t cand_merged;      /* candidates read by the merges */
    uint64_t pool_entries_merged; /* pool entries rewritten by the merges */
    uint64_t tree_attached;    /* edges added by tree_grow to reach unreached nodes */
    double iter_join_ms[KCNA_MAX_ITERS];   /* device time of each NN-descent join */
    double iter_merge_ms[KCNA_MAX_ITERS];  /* device time of each NN-descent merge */
    uint64_t iter_cand[KCNA_MAX_ITERS];    /* candidates merged in each NN-descent iteration */
    uint64_t iter_inserted[KCNA_MAX_ITERS]; /* of which inserted into pools */
    /* learned seed (kcna_params.learned_seed = 1) */
    double seed_train_ms;      /* subsample NN-descent + encoder training */
    double seed_total_ms;      /* training + encoding + hashing + initial pools */
    float seed_loss_first, seed_loss_last; /* triplet loss of the first and last training batch */
    float seed_input_scale;    /* 1 / RMS of the rows, folded into the first layer */
    float seed_recall;         /* control recall@K of the seeded pools, before the first join */
    uint64_t seed_comps;       /* distance evaluations of the initial pools */
    uint32_t bf16_rows;        /* 1: BF16 mode read an exact BF16 copy of the rows */
    uint32_t gram_tc;          /* local join on tensor-core Gram tiles: 1 exact (integer rows,
                                  squared norms < 2^23), 2 screening of rows rounded to BF16 with
                                  FP32 recompute of the emitted pairs; d <= 128, a multiple of 8 */
    uint32_t prune_tc;         /* 1: the occlusion prunes ran on tensor-core Gram tiles (Gram-exact rows);
                                  2: the tau-MNG prunes screened float rows on FP8 E4M3 Gram tiles
                                  (d >= 256), undecided pairs recomputed in FP32 */
    uint64_t prune_exact;      /* pairs of the FP8-screened prunes recomputed in FP32 */
    uint64_t prune_skipped;    /* node prunes skipped: the node's first search_K pool entries (ids,
                                  distances) and their count were those of the previous prune of
                                  the build, whose kept list was reused */
} kcna_stats;

typedef struct kcna_ctx kcna_ctx;

/* Context on CUDA device `device`.  Replaces KGraph::create (src/kgraph.cpp:3968-3971). */
kcna_status kcna_create(kcna_ctx **out, int device);
void kcna_destroy(kcna_ctx *ctx);
const char *kcna_last_error(const kcna_ctx *ctx);
const char *kcna_version(void); /* replaces KGraph::version (src/kgraph.cpp:3973) */

/* Copies n rows of d floats (row pitch stride_bytes) from HOST memory into the
 * context.  Replaces constructing MatrixOracle over a Matrix<float>
 * (src/kgraph-data.h:349-384; src/fastnsg.cpp:193). */
kcna_status kcna_upload(kcna_ctx *ctx, const float *rows, uint32_t n, uint32_t d, uint64_t stride_bytes);
/* Same, from DEVICE memory of the context's device (no host copy). */
kcna_status kcna_upload_device(kcna_ctx *ctx, const float *dev_rows, uint32_t n, uint32_t d, uint64_t stride_bytes);
/* Loads an lshkit float file (u32 header {4, rows, cols}, then the rows; the
 * row count follows from the file size) straight into the context: the file
 * is mapped and streamed through two pinned 64 MiB staging buffers.  Replaces
 * Matrix::load_lshkit + MatrixOracle (src/kgraph-data.h:161-177, 262-274). */
kcna_status kcna_upload_lshkit(kcna_ctx *ctx, const char *path);
/* Restricts every following call to the first n_prefix rows.
 * Replaces IndexOracle::set_size (src/kgraph.h:80, src/kgraph-data.h:372-382). */
kcna_status kcna_set_size(kcna_ctx *ctx, uint32_t n_prefix);

/* Exact k-NN of m base rows (ids) against all rows, self excluded; ties broken by
 * lower id.  Replaces LinearSearch (src/kgraph.cpp:309-330).  Host outputs m*k. */
kcna_status kcna_knn_exact(kcna_ctx *ctx, const uint32_t *ids, uint32_t m, uint32_t k,
                           uint32_t *out_ids, float *out_dists);
/* Exact k-NN of m host query vectors (pitch q_stride_bytes) against all rows.
 * Replaces SearchOracle::search (src/kgraph.cpp:332-361). */
kcna_status kcna_knn_queries(kcna_ctx *ctx, const float *queries, uint32_t m, uint64_t q_stride_bytes,
                             uint32_t k, uint32_t *out_ids, float *out_dists);

/* Full build of one graph kind: NN-descent, then loop_i+1 rounds of
 * {prune+link, entry point, [tree_grow], UpdateNhoods, [P2K refinement]}.
 * Replaces KGraph::buildFastNSG / buildFastTauMNG / buildFastAlphaPG
 * (src/kgraph.h:230-232; src/kgraph.cpp:3796-3966) and the per-layer part of
 * buildFastHNSW (src/kgraph.h:233; src/kgraph.cpp:3720-3795). */
kcna_status kcna_build(kcna_ctx *ctx, const kcna_params *params, kcna_kind kind, kcna_stats *stats);

/* NN-descent only (the KGraphConstructor constructor, src/kgraph.cpp:1281-1459),
 * leaving the pools in the context. */
kcna_status kcna_nndescent(kcna_ctx *ctx, const kcna_params *params, kcna_stats *stats);

/* Graph after a build: ids is n*width (rows padded with 0xFFFFFFFF), degrees n.
 * Pass NULL ids to query width only.  Replaces reading nn_nsg as SaveNsg does
 * (src/kgraph.cpp:1704-1724) and SwapPGraph (:2296-2311). */
kcna_status kcna_get_graph(kcna_ctx *ctx, uint32_t *ids, uint32_t *degrees, uint32_t *ep, uint32_t *width);

/* Candidate pools (sorted by distance): ids/dists n*cap, counts n.  cap must be
 * >= the pool capacity reported by kcna_pool_capacity. */
kcna_status kcna_pool_capacity(kcna_ctx *ctx, uint32_t *cap);
kcna_status kcna_get_pools(kcna_ctx *ctx, uint32_t *ids, float *dists, uint32_t *counts, uint32_t cap);
/* Installs caller pools (each sorted ascending by distance, no duplicate ids)
 * so that prune/link can be run on an identical input KNN graph. */
kcna_status kcna_set_pools(kcna_ctx *ctx, const kcna_params *params, const uint32_t *ids, const float *dists,
                           const uint32_t *counts, uint32_t cap);

/* Occlusion prune of every pool into the graph (kind NSG/HNSW_LAYER: RNG,
 * TAUMNG: tau, ALPHAPG: angle).  Replaces nsg_sync_prune (src/kgraph.cpp:1809-1851),
 * taumg_sync_prune (:2833-2876) and alphapg_sync_prune (:3157-3203).
 * Kind CAGRA: the rank prune of BuildCagra (src/kgraph.cpp:2665-2829) over the
 * first K pool entries, about K / 2 edges per node (width >= K / 2 + 1);
 * 2 <= K <= min(pool capacity, 1024). */
kcna_status kcna_prune(kcna_ctx *ctx, const kcna_params *params, kcna_kind kind);
/* Prune + reverse-edge insert + re-prune of over-full nodes.  Replaces
 * nsg_Link / taumg_Link / alphapg_Link (src/kgraph.cpp:2087-2143, 3085-3141, 3424-3480). */
kcna_status kcna_link(kcna_ctx *ctx, const kcna_params *params, kcna_kind kind);
/* Per-node pool search of loop `loopcount` (>= 1): every node's pool is the
 * beam of a greedy search over the context graph, expanding the entries at
 * positions < min(search_L + (loopcount - 1) * step, MAXL).  Replaces inSearch /
 * poolSearch (src/kgraph.cpp:3667-3688, 2340-2414); kcna_build runs it between
 * prune loops when params->refine is KCNA_REFINE_POOL_SEARCH.  comps (may be
 * NULL) receives the distance evaluations. */
kcna_status kcna_pool_search(kcna_ctx *ctx, const kcna_params *params, uint32_t loopcount, uint64_t *comps);
/* One refinement step of the pools between prune loops, as kcna_build runs it
 * after the prune loop that made the context graph: UpdateNhoods marks every
 * graph edge new when loopcount is 1, else new iff it is absent from the graph
 * of the previous refinement step (src/kgraph.cpp:3537-3584); then the pools
 * are refined over the graph for loop `loopcount` (>= 1): BridgeView
 * (src/kgraph.cpp:2478-2663), or the per-node pool search when params->refine
 * is KCNA_REFINE_POOL_SEARCH.  Needs pools (a build or kcna_set_pools) and a
 * graph (a build or kcna_set_graph).  comps (may be NULL) receives the
 * distance evaluations of the refinement's joins. */
kcna_status kcna_refine_pools(kcna_ctx *ctx, const kcna_params *params, uint32_t loopcount, uint64_t *comps);
/* The isnew flag of every graph edge as UpdateNhoods last set it (n*width
 * bytes, 1 = new; replaces reading nn_nsg[j].isnew, src/kgraph.cpp:3548-3555). */
kcna_status kcna_get_edge_isnew(kcna_ctx *ctx, uint8_t *isnew);
/* Installs a caller graph (ids n*width padded with 0xFFFFFFFF, degrees n). */
kcna_status kcna_set_graph(kcna_ctx *ctx, const uint32_t *ids, const uint32_t *degrees, uint32_t width, uint32_t ep);

/* Greedy beam search of m host queries over the context graph, beam width L,
 * starting from init_ids (m*L host ids, or NULL: entry point + its graph
 * neighbours).  Outputs the best k (m*k).  Replaces get_neighbors
 * (src/kgraph.cpp:1560-1623) and serves the query-time recall@10 evaluator. */
kcna_status kcna_search(kcna_ctx *ctx, const float *queries, uint32_t m, uint64_t q_stride_bytes,
                        const uint32_t *init_ids, uint32_t L, uint32_t k,
                        uint32_t *out_ids, float *out_dists);

/* Number of kernels this context has launched so far. */
uint64_t kcna_kernel_launches(const kcna_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), so that a caller can order its
 * own work or timing events against the library's kernels. */
void *kcna_stream(const kcna_ctx *ctx);

/* Exact k-NN that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc where they need neighbours: code that
 * runs under a fixed memory budget and hands out device memory only through its
 * own arena, or a plugin called from inside a host framework that owns the
 * device allocator.  Base rows, queries and outputs are caller-owned DEVICE
 * buffers (base n x d, pitch base_stride_bytes; queries m x d, pitch
 * q_stride_bytes; outputs m x k ids and squared L2 distances, ties broken by
 * the lower id, identical to kcna_knn_queries).  The only working memory is one
 * static device array of KCNA_NOALLOC_SCRATCH_BYTES (16 MiB) inside the
 * library, which every GPU that loads the library holds until the process
 * exits; queries are processed in batches of (16 MiB - 256 B) / (4 n) rows.
 * Limits (KCNA_E_ARG otherwise): n * 4 <= 16 MiB - 256 B (n <= 4,194,240),
 * 1 <= k <= min(n, 1024), d a multiple of 4, strides multiples of 16 bytes,
 * 16-byte aligned pointers.  KCNA_E_LIMIT: more than 1024 base rows tie at the
 * k-th distance of some query (a property of the data, e.g. many duplicate
 * rows); the outputs are then unspecified and the next call starts clean.
 * KCNA_E_CUDA: a CUDA call failed, or a runtime error was already pending on
 * this host thread when the call began (it is left pending for its owner).
 * Runs on `stream` (a cudaStream_t, NULL = the legacy default stream) of the
 * current device, copies a 4-byte status word to a host stack variable and
 * synchronises the stream (cudaStreamSynchronize) before returning, so no
 * call may be made while a stream of the device is being captured into a CUDA
 * graph.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current.
 * All calls share the one array: calls whose kernels overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 * Each call clears the array's error word itself. */
#define KCNA_NOALLOC_SCRATCH_BYTES (16u << 20)
kcna_status kcna_knn_queries_noalloc(const float *d_base, uint32_t n, uint32_t d, uint64_t base_stride_bytes,
                                     const float *d_queries, uint32_t m, uint64_t q_stride_bytes, uint32_t k,
                                     uint32_t *d_out_ids, float *d_out_dists, void *stream);

/* C[M x N] (FP32, row-major, pitch ldc) = A * B^T on the tcgen05 tensor cores
 * in BF16 with FP32 accumulation.  Element (r, k) of A is A[r * lda + k]
 * (a_trans = 1: A[k * lda + r]); a_fp32 selects FP32 (converted to BF16 with
 * round-to-nearest-even) or BF16 storage; likewise B.  Device pointers, runs
 * on `stream` and synchronises it.  No counterpart in the reference: the
 * product primitive of the learned-seed encoder and the BF16 distance screen. */
kcna_status kcna_gemm_bf16(const void *A, int64_t lda, int a_fp32, int a_trans, const void *B, int64_t ldb,
                           int b_fp32, int b_trans, float *C, int64_t ldc, int M, int N, int K, void *stream);

/* One forward + backward pass of the learned-seed encoder, for gradient checks.
 * No counterpart in the reference.  rows = 3B host rows of dimension d laid
 * out as [anchors | positives | negatives]; W1 256 x d, b1 256, W2 64 x 256,
 * b2 64 (host, FP32, row-major).  Outputs (host): the mean triplet loss and the
 * gradients of every parameter.  The products run in BF16 on the tensor cores
 * with FP32 accumulation, as in training. */
kcna_status kcna_encoder_grads(kcna_ctx *ctx, const float *rows, uint32_t n_rows, uint32_t d, const float *W1,
                               const float *b1, const float *W2, const float *b2, float margin, float *loss,
                               float *dW1, float *db1, float *dW2, float *db2);

/* Writes the graph in the NSG/efanna format written by SaveNsg
 * (src/kgraph.cpp:1704-1724): u32 width, u32 ep, per node u32 GK + GK u32 ids. */
kcna_status kcna_write_nsg(kcna_ctx *ctx, const char *path);
/* Same file, written on a host thread after one device-to-host snapshot of the
 * graph, so the caller can go on; one write in flight per context.
 * kcna_wait_writes joins it and returns its outcome (KCNA_E_IO on failure);
 * kcna_destroy joins it too. */
kcna_status kcna_write_nsg_async(kcna_ctx *ctx, const char *path);
kcna_status kcna_wait_writes(kcna_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* KCNA_H */
