// kcna_api.cu - C ABI, context and build driver of the GB300 FastKCNA library.
//
// The build driver follows KGraphImpl::buildFastNSG / buildFastTauMNG /
// buildFastAlphaPG (src/kgraph.cpp:3796-3966) and the per-layer part of
// buildFastHNSW (:3720-3795): NN-descent, evaluate, then loop_i+1 rounds of
// {link, ComputeEp, [tree_grow], UpdateNhoods} with a P2K refinement
// (BridgeView) and evaluate between rounds.  All compute runs in the CUDA
// kernels of kcna_knn.cu, kcna_nnd.cu and kcna_graph.cu; the host only
// sequences phases, reads counters and moves data across the boundary.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>
#include <set>
#include <vector>

#include <cuda_bf16.h>

#include "kcna_common.cuh"
#include "kcna_internal.h"

#ifndef KCNA_VERSION_STRING
#define KCNA_VERSION_STRING "kcna-gb300 0.1 (sm_103a)"
#endif

double kcna_now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

kcna_status kcna_fail(kcna_ctx *c, kcna_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

kcna_status kcna_cuda_check(kcna_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return KCNA_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return kcna_fail(c, KCNA_E_OOM, m);
    return kcna_fail(c, KCNA_E_CUDA, m);
}

kcna_status kcna_check_device_err(kcna_ctx *c, const char *phase) {
    int h = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&h, c->d_err, 4, cudaMemcpyDeviceToHost, c->stream), "err d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "err sync"));
    if (h == 0) return KCNA_OK;
    cudaMemsetAsync(c->d_err, 0, 4, c->stream);
    cudaStreamSynchronize(c->stream);
    const char *what = h == 1 ? "index outside its buffer (access skipped)"
                       : h == 2 ? "bounded wait gave up"
                       : h == 3 ? "graph row ran out of slots"
                       : h == 4 ? "more than 1024 rows tie at the k-th distance"
                                : "unknown";
    const kcna_status st = h == 2 ? KCNA_E_TIMEOUT : h == 4 ? KCNA_E_LIMIT : KCNA_E_CUDA;
    return kcna_fail(c, st, std::string(phase) + ": device error: " + what);
}

kcna_status kcna_phase_begin(kcna_ctx *c) {
    c->launches_at_begin = c->launches;
    return kcna_cuda_check(c, cudaEventRecord(c->ev0, c->stream), "event record");
}

kcna_status kcna_phase_end(kcna_ctx *c, int phase) {
    KCNA_TRY(kcna_cuda_check(c, cudaEventRecord(c->ev1, c->stream), "event record"));
    KCNA_TRY(kcna_cuda_check(c, cudaEventSynchronize(c->ev1), "event sync"));
    float ms = 0.f;
    KCNA_TRY(kcna_cuda_check(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event elapsed"));
    if (phase >= 0 && phase < KCNA_NUM_PHASES) {
        c->phase_ms[phase] += ms;
        c->phase_launches[phase] += c->launches - c->launches_at_begin;
    }
    return KCNA_OK;
}

static void reset_phase_stats(kcna_ctx *c) {
    for (int i = 0; i < KCNA_NUM_PHASES; ++i) {
        c->phase_ms[i] = 0;
        c->phase_launches[i] = 0;
    }
    c->join_rows = c->cand_emitted = c->cand_merged = c->pool_entries_merged = c->tree_attached = 0;
    c->prune_exact = 0;
    c->prune_skipped = 0;
}

static void copy_phase_stats(const kcna_ctx *c, kcna_stats *st) {
    for (int i = 0; i < KCNA_NUM_PHASES; ++i) {
        st->phase_ms[i] = c->phase_ms[i];
        st->phase_launches[i] = c->phase_launches[i];
    }
    st->join_rows = c->join_rows;
    st->cand_emitted = c->cand_emitted;
    st->cand_merged = c->cand_merged;
    st->pool_entries_merged = c->pool_entries_merged;
    st->tree_attached = c->tree_attached;
    st->prune_exact = c->prune_exact;
    st->prune_skipped = c->prune_skipped;
}

kcna_status kcna_dev_malloc(kcna_ctx *c, size_t bytes, void **out, const char *what) {
    *out = nullptr;
    // smallest cached block that holds `bytes` without wasting more than half of it
    auto it = c->free_blocks.lower_bound(bytes);
    if (it != c->free_blocks.end() && it->first <= 2 * bytes + (1u << 20)) {
        *out = it->second;
        c->free_blocks.erase(it);
        return KCNA_OK;
    }
    cudaError_t e = cudaMalloc(out, bytes);
    if (e == cudaErrorMemoryAllocation && !c->free_blocks.empty()) {
        (void)cudaGetLastError();
        kcna_release_all(c);
        e = cudaMalloc(out, bytes);
    }
    if (e != cudaSuccess) {
        *out = nullptr;
        (void)cudaGetLastError();
        return kcna_fail(c, KCNA_E_OOM, std::string("cudaMalloc failed for ") + what);
    }
    c->block_bytes[*out] = bytes;
    return KCNA_OK;
}

void kcna_release(kcna_ctx *c, void *p) {
    if (!p) return;
    auto it = c->block_bytes.find(p);
    if (it == c->block_bytes.end()) {
        cudaFree(p);
        return;
    }
    c->free_blocks.emplace(it->second, p);
}

void kcna_release_all(kcna_ctx *c) {
    for (auto &b : c->free_blocks) {
        c->block_bytes.erase(b.second);
        cudaFree(b.second);
    }
    c->free_blocks.clear();
}

static kcna_status grow(kcna_ctx *c, void **p, size_t *cur, size_t bytes) {
    if (*cur >= bytes && *p) return KCNA_OK;
    if (*p) kcna_release(c, *p);
    *p = nullptr;
    *cur = 0;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        *p = nullptr;
        return kcna_fail(c, KCNA_E_OOM, "scratch allocation failed");
    }
    *cur = bytes;
    return KCNA_OK;
}
kcna_status kcna_scratch(kcna_ctx *c, size_t bytes, void **out) {
    KCNA_TRY(grow(c, &c->scratch, &c->scratch_bytes, bytes));
    *out = c->scratch;
    return KCNA_OK;
}
kcna_status kcna_scratch2(kcna_ctx *c, size_t bytes, void **out) {
    KCNA_TRY(grow(c, &c->scratch2, &c->scratch2_bytes, bytes));
    *out = c->scratch2;
    return KCNA_OK;
}

void kcna_log(kcna_ctx *c, const kcna_params *p, const char *fmt, ...) {
    (void)c;
    if (!p || !p->verbosity) return;
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[kcna] ");
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
}

static void free_state(kcna_ctx *c) {
    void *bufs[] = {c->pool, c->pool_cnt, c->radius, c->M, c->radiusM, c->found, c->fwd_new, c->fwd_new_cnt,
                    c->fwd_old, c->fwd_old_cnt, c->rnew, c->rnew_cnt, c->rold, c->rold_cnt, c->cand, c->cand_cnt,
                    c->g_ids, c->g_deg, c->g_old, c->g_old_deg, c->g_dist, c->g_isnew, c->d_controls,
                    c->d_control_knn, c->big_list, c->big_cnt, c->inc_snap, c->inc_cnt, c->inc_ids, c->inc_deg,
                    c->inc_list, c->inc_dist};
    for (void *b : bufs)
        if (b) kcna_release(c, b);
    c->pool = nullptr;
    c->pool_cnt = nullptr;
    c->radius = nullptr;
    c->M = nullptr;
    c->radiusM = nullptr;
    c->found = nullptr;
    c->fwd_new = c->fwd_new_cnt = c->fwd_old = c->fwd_old_cnt = nullptr;
    c->rnew = c->rnew_cnt = c->rold = c->rold_cnt = nullptr;
    c->cand = nullptr;
    c->cand_cnt = nullptr;
    c->big_list = c->big_cnt = nullptr;
    c->g_ids = c->g_deg = c->g_old = c->g_old_deg = nullptr;
    c->g_dist = nullptr;
    c->g_isnew = nullptr;
    c->d_controls = c->d_control_knn = nullptr;
    c->inc_snap = nullptr;
    c->inc_cnt = c->inc_ids = c->inc_deg = c->inc_list = nullptr;
    c->inc_dist = nullptr;
    c->inc_valid = false; // a build never reuses an earlier build's prune
    c->W = 0;
    c->cap = 0;
    c->has_graph = c->has_pools = false;
}

static kcna_status bind(kcna_ctx *c) { return kcna_cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice"); }

// A float is exactly representable in BF16 when its low 16 bits are zero.
__global__ void bf16_inexact_kernel(const uint32_t *__restrict__ x, uint64_t n, unsigned long long *inexact) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long bad = 0;
    for (; t < n; t += (uint64_t)gridDim.x * blockDim.x) bad += (x[t] & 0xFFFFu) ? 1 : 0;
    bad = kcna_warp_sum(bad);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(inexact, bad);
}
__global__ void bf16_copy_kernel(const uint32_t *__restrict__ x, uint64_t n, uint16_t *__restrict__ out) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (uint16_t)(x[t] >> 16);
}

// Gram-exact check: every value an integer (BF16 exactness is checked
// before), squared norms |x|^2 into norms[] (exact for integer rows), the
// largest one and whether any value is negative.  Warp per row.
__global__ void gram_check_kernel(const float *__restrict__ X, uint32_t n, uint32_t ld, float *__restrict__ norms,
                                  unsigned long long *nonint, unsigned *max_bits, unsigned long long *negative) {
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float acc = 0.f;
    bool bad = false, neg = false;
    for (uint32_t k = lane; k < ld; k += 32) {
        const float x = X[row * ld + k];
        bad |= x != rintf(x);
        neg |= x < 0.f;
        acc = fmaf(x, x, acc);
    }
    acc = kcna_warp_sum(acc);
    bad = __any_sync(KCNA_FULL, bad);
    neg = __any_sync(KCNA_FULL, neg);
    if (lane == 0) {
        norms[row] = acc;
        if (bad) atomicAdd(nonint, 1ull);
        if (neg) atomicAdd(negative, 1ull);
        atomicMax(max_bits, __float_as_uint(acc));
    }
}

static void release_row_copies(kcna_ctx *c) {
    if (c->Xh) kcna_release(c, c->Xh);
    if (c->norms) kcna_release(c, c->norms);
    if (c->Xq) kcna_release(c, c->Xq);
    if (c->qmeta) kcna_release(c, c->qmeta);
    c->Xh = nullptr;
    c->norms = nullptr;
    c->Xq = nullptr;
    c->qmeta = nullptr;
    c->gram_exact = c->bf16_exact = c->bf16_screen = c->fp8_screen = false;
}

// BF16 copy rounded to nearest (even) and the squared norms of the rounded
// rows, for screening inexact data; warp per row.
__global__ void bf16_round_kernel(const float *__restrict__ X, uint32_t n, uint32_t ld, uint16_t *__restrict__ Xh,
                                  float *__restrict__ norms) {
    const uint64_t row = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float acc = 0.f;
    for (uint32_t k = lane; k < ld; k += 32) {
        const __nv_bfloat16 b = __float2bfloat16_rn(X[row * ld + k]);
        Xh[row * ld + k] = *reinterpret_cast<const uint16_t *>(&b);
        const float v = __bfloat162float(b);
        acc = fmaf(v, v, acc);
    }
    acc = kcna_warp_sum(acc);
    if (lane == 0) norms[row] = acc;
}

// BF16 mode: when every value of the rows is exactly representable in BF16,
// kernels read a BF16 copy (same floats, half the bytes).  When the rows are
// moreover integers with squared norms below 2^23 (and d <= 128, a multiple of
// 8), the local join runs on tensor-core Gram tiles whose distances are exact.
// Returns whether the copy is in use and whether the Gram tiles are.
static kcna_status prepare_rows(kcna_ctx *c, const kcna_params *p, uint32_t *used, uint32_t *gram = nullptr) {
    *used = 0;
    if (gram) *gram = 0;
    release_row_copies(c);
    if (!p || p->screen != KCNA_SCREEN_BF16) return KCNA_OK;
    const uint64_t n = (uint64_t)c->n_total * c->ld;
    KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->counters + 40, 0, 4 * 8, c->stream), "memset"));
    bf16_inexact_kernel<<<std::max(1, c->num_sms) * 8, 256, 0, c->stream>>>(reinterpret_cast<const uint32_t *>(c->X), n,
                                                                             c->counters + 40);
    KCNA_LAUNCHED(c);
    unsigned long long bad = 0;
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(&bad, c->counters + 40, 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "bf16 check"));
    if (bad) { // inexact data: FP32 rows everywhere; the join screens on a rounded copy
        // high dimension: the tau-MNG prune screens on FP8 E4M3 codes instead
        if (c->d >= 256) return kcna_fp8_rows(c);
        if ((c->ld & 7u) || c->ld > 128) return KCNA_OK;
        KCNA_TRY(kcna_alloc(c, &c->Xh, n, "bf16 rows (rounded)"));
        KCNA_TRY(kcna_alloc(c, &c->norms, c->n_total, "row norms"));
        bf16_round_kernel<<<kcna_div_up((uint64_t)c->n_total * 32, 256), 256, 0, c->stream>>>(c->X, c->n_total, c->ld,
                                                                                              c->Xh, c->norms);
        KCNA_LAUNCHED(c);
        c->bf16_screen = true;
        if (gram) *gram = 2;
        return kcna_cuda_check(c, cudaGetLastError(), "bf16 round");
    }
    KCNA_TRY(kcna_alloc(c, &c->Xh, n, "bf16 rows"));
    c->bf16_exact = true;
    bf16_copy_kernel<<<kcna_div_up(n, 256), 256, 0, c->stream>>>(reinterpret_cast<const uint32_t *>(c->X), n, c->Xh);
    KCNA_LAUNCHED(c);
    KCNA_TRY(kcna_cuda_check(c, cudaGetLastError(), "bf16 copy"));
    *used = 1;
    if ((c->ld & 7u) || c->ld > 128) return KCNA_OK;
    KCNA_TRY(kcna_alloc(c, &c->norms, c->n_total, "row norms"));
    unsigned *max_bits = reinterpret_cast<unsigned *>(c->counters + 42);
    gram_check_kernel<<<kcna_div_up((uint64_t)c->n_total * 32, 256), 256, 0, c->stream>>>(c->X, c->n_total, c->ld,
                                                                                          c->norms, c->counters + 41,
                                                                                          max_bits, c->counters + 43);
    KCNA_LAUNCHED(c);
    unsigned long long h[3] = {};
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(h, c->counters + 41, 24, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "gram check"));
    float maxn = 0.f;
    const unsigned mb = (unsigned)(h[1] & 0xFFFFFFFFull);
    memcpy(&maxn, &mb, 4);
    // every distance, partial sum and |x|^2 - 2<x,y> below 2^24: with non-negative
    // values |x - y|^2 <= |x|^2 + |y|^2 < 2^24; with negative ones |x|, |y| < 2^11
    if (h[0] == 0 && maxn < (h[2] ? 4194304.f : 8388608.f)) {
        c->gram_exact = true;
        if (gram) *gram = 1;
    } else {
        kcna_release(c, c->norms);
        c->norms = nullptr;
    }
    return KCNA_OK;
}

kcna_status kcna_rows_reset(kcna_ctx *c, uint32_t n, uint32_t d) {
    if (n < 2 || d == 0 || n > KCNA_MAX_ID) return kcna_fail(c, KCNA_E_ARG, "upload: need n >= 2, d >= 1, n < 2^30");
    KCNA_TRY(bind(c));
    free_state(c);
    if (c->X) kcna_release(c, c->X);
    c->X = nullptr;
    release_row_copies(c);
    c->d = d;
    c->ld = (d + 3) & ~3u;
    c->n_total = c->n = n;
    KCNA_TRY(kcna_alloc(c, &c->X, (size_t)n * c->ld, "rows"));
    if (c->ld != d) KCNA_TRY(kcna_cuda_check(c, cudaMemsetAsync(c->X, 0, (size_t)n * c->ld * 4, c->stream), "memset"));
    return KCNA_OK;
}

extern "C" {

void kcna_params_default(kcna_params *p) {
    memset(p, 0, sizeof *p);
    p->K = 25;
    p->L = 100;
    p->S = 10;
    p->R = 100;
    p->iterations = 30;
    p->controls = 100;
    p->seed = 2024;
    p->nthreads = 40;
    p->delta = 0.002f;
    p->recall = 0.95f;
    p->nsg_R = 50;
    p->search_L = 40;
    p->search_K = 500;
    p->step = 10;
    p->massq_S = 10;
    p->loop_i = 2;
    p->tau = 0.f;
    p->angle = 60.f;
}

const char *kcna_version(void) { return KCNA_VERSION_STRING; }

kcna_status kcna_create(kcna_ctx **out, int device) {
    if (!out) return KCNA_E_ARG;
    *out = nullptr;
    kcna_ctx *c = new kcna_ctx();
    c->device = device;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || device < 0 || device >= count) {
        (void)cudaGetLastError();
        delete c;
        return KCNA_E_CUDA;
    }
    kcna_status s = bind(c);
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device), "attr");
    if (s == KCNA_OK) s = kcna_alloc(c, &c->d_err, 1, "error word");
    if (s == KCNA_OK) s = kcna_alloc(c, &c->counters, 64, "counters");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaMemset(c->d_err, 0, 4), "memset");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaEventCreate(&c->ev0), "event");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaEventCreate(&c->ev1), "event");
    if (s != KCNA_OK) {
        kcna_destroy(c);
        return s;
    }
    *out = c;
    return KCNA_OK;
}

void kcna_destroy(kcna_ctx *c) {
    if (!c) return;
    if (c->writer.joinable()) c->writer.join();
    if (c->seed_sub) kcna_destroy(c->seed_sub);
    c->seed_sub = nullptr;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_state(c);
    if (c->X) kcna_release(c, c->X);
    release_row_copies(c);
    if (c->scratch) kcna_release(c, c->scratch);
    if (c->scratch2) kcna_release(c, c->scratch2);
    if (c->d_err) kcna_release(c, c->d_err);
    if (c->counters) kcna_release(c, c->counters);
    kcna_release_all(c);
    for (auto &b : c->block_bytes) cudaFree(b.first); // blocks still held by no pointer of the context
    c->block_bytes.clear();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *kcna_last_error(const kcna_ctx *c) { return c ? c->err.c_str() : "no context"; }

uint64_t kcna_kernel_launches(const kcna_ctx *c) { return c ? c->launches : 0; }

void *kcna_stream(const kcna_ctx *c) { return c ? (void *)c->stream : nullptr; }

static kcna_status upload(kcna_ctx *c, const float *rows, uint32_t n, uint32_t d, uint64_t stride, cudaMemcpyKind kind) {
    if (!c) return KCNA_E_ARG;
    if (!rows || stride < (uint64_t)d * 4)
        return kcna_fail(c, KCNA_E_ARG, "upload: need rows, n >= 2, d >= 1, stride >= 4*d, n < 2^30");
    KCNA_TRY(kcna_rows_reset(c, n, d));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpy2DAsync(c->X, (size_t)c->ld * 4, rows, stride, (size_t)d * 4, n, kind, c->stream),
                             "upload copy"));
    return kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "upload sync");
}

kcna_status kcna_upload(kcna_ctx *c, const float *rows, uint32_t n, uint32_t d, uint64_t stride_bytes) {
    return upload(c, rows, n, d, stride_bytes, cudaMemcpyHostToDevice);
}
kcna_status kcna_upload_device(kcna_ctx *c, const float *rows, uint32_t n, uint32_t d, uint64_t stride_bytes) {
    return upload(c, rows, n, d, stride_bytes, cudaMemcpyDeviceToDevice);
}

kcna_status kcna_set_size(kcna_ctx *c, uint32_t n_prefix) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "set_size: no rows");
    if (n_prefix < 2) return kcna_fail(c, KCNA_E_ARG, "set_size: need at least 2 rows");
    KCNA_TRY(bind(c));
    free_state(c);
    c->n = std::min(n_prefix, c->n_total); // IndexOracle::set_size clamps (src/kgraph-data.h:372-382)
    return KCNA_OK;
}

static kcna_status to_device_rows(kcna_ctx *c, const float *q, uint32_t m, uint64_t stride, float **out) {
    float *dq = nullptr;
    KCNA_TRY(kcna_alloc(c, &dq, (size_t)m * c->ld, "query rows"));
    kcna_status s = KCNA_OK;
    if (c->ld != c->d) s = kcna_cuda_check(c, cudaMemsetAsync(dq, 0, (size_t)m * c->ld * 4, c->stream), "memset");
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpy2DAsync(dq, (size_t)c->ld * 4, q, stride, (size_t)c->d * 4, m,
                                                 cudaMemcpyHostToDevice, c->stream),
                            "query copy");
    if (s != KCNA_OK) {
        kcna_release(c, dq);
        return s;
    }
    *out = dq;
    return KCNA_OK;
}

kcna_status kcna_knn_exact(kcna_ctx *c, const uint32_t *ids, uint32_t m, uint32_t k, uint32_t *out_ids,
                           float *out_dists) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "knn_exact: no rows");
    if (!ids || !out_ids || !out_dists || m == 0) return kcna_fail(c, KCNA_E_ARG, "knn_exact: null argument");
    for (uint32_t i = 0; i < m; ++i)
        if (ids[i] >= c->n) return kcna_fail(c, KCNA_E_ARG, "knn_exact: id out of range");
    KCNA_TRY(bind(c));
    uint32_t *did = nullptr, *oid = nullptr;
    float *rows = nullptr, *od = nullptr;
    kcna_status s = kcna_alloc(c, &did, m, "ids");
    if (s == KCNA_OK) s = kcna_alloc(c, &rows, (size_t)m * c->ld, "rows");
    if (s == KCNA_OK) s = kcna_alloc(c, &oid, (size_t)m * k, "out ids");
    if (s == KCNA_OK) s = kcna_alloc(c, &od, (size_t)m * k, "out dists");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaMemcpyAsync(did, ids, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    if (s == KCNA_OK) s = kcna_gather_rows(c, did, m, rows);
    if (s == KCNA_OK) s = kcna_knn_device(c, rows, m, did, k, oid, od);
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_ids, oid, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_dists, od, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "knn sync");
    kcna_release(c, did);
    kcna_release(c, rows);
    kcna_release(c, oid);
    kcna_release(c, od);
    return s == KCNA_OK ? kcna_check_device_err(c, "knn_exact") : s;
}

kcna_status kcna_knn_queries(kcna_ctx *c, const float *queries, uint32_t m, uint64_t q_stride, uint32_t k,
                             uint32_t *out_ids, float *out_dists) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "knn_queries: no rows");
    if (!queries || !out_ids || !out_dists || m == 0 || q_stride < (uint64_t)c->d * 4)
        return kcna_fail(c, KCNA_E_ARG, "knn_queries: bad argument");
    KCNA_TRY(bind(c));
    float *dq = nullptr, *od = nullptr;
    uint32_t *oid = nullptr;
    kcna_status s = to_device_rows(c, queries, m, q_stride, &dq);
    if (s == KCNA_OK) s = kcna_alloc(c, &oid, (size_t)m * k, "out ids");
    if (s == KCNA_OK) s = kcna_alloc(c, &od, (size_t)m * k, "out dists");
    if (s == KCNA_OK) s = kcna_knn_device(c, dq, m, nullptr, k, oid, od);
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_ids, oid, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_dists, od, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "knn sync");
    kcna_release(c, dq);
    kcna_release(c, oid);
    kcna_release(c, od);
    return s == KCNA_OK ? kcna_check_device_err(c, "knn_queries") : s;
}

kcna_status kcna_nndescent(kcna_ctx *c, const kcna_params *p, kcna_stats *st) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "nndescent: no rows");
    if (!p) return kcna_fail(c, KCNA_E_ARG, "nndescent: null params");
    KCNA_TRY(bind(c));
    kcna_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof *st);
    free_state(c);
    reset_phase_stats(c);
    c->t0 = kcna_now();
    KCNA_TRY(prepare_rows(c, p, &st->bf16_rows, &st->gram_tc));
    KCNA_TRY(kcna_nndescent_run(c, p, st));
    float r = 0;
    KCNA_TRY(kcna_control_recall(c, c->cap, &r));
    st->loop_recall[0] = r;
    st->nndescent_time = kcna_now() - c->t0;
    st->total_time = st->nndescent_time;
    copy_phase_stats(c, st);
    return kcna_check_device_err(c, "nndescent");
}

static kcna_status degree_stats(kcna_ctx *c, kcna_stats *st) {
    std::vector<uint32_t> deg(c->n);
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(deg.data(), c->g_deg, (size_t)c->n * 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync"));
    uint64_t sum = 0;
    uint32_t mx = 0, mn = ~0u;
    for (uint32_t d : deg) {
        sum += d;
        mx = std::max(mx, d);
        mn = std::min(mn, d);
    }
    c->width = mx;
    st->width = mx;
    st->max_degree = mx;
    st->min_degree = mn;
    st->aod = (uint32_t)(sum / std::max<uint32_t>(1, c->n)); // CalculateNSG (src/kgraph.cpp:2273-2293)
    st->ep = c->ep;
    return KCNA_OK;
}

kcna_status kcna_build(kcna_ctx *c, const kcna_params *p, kcna_kind kind, kcna_stats *st) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "build: no rows");
    if (!p) return kcna_fail(c, KCNA_E_ARG, "build: null params");
    if (kind != KCNA_NSG && kind != KCNA_HNSW_LAYER && kind != KCNA_TAUMNG && kind != KCNA_ALPHAPG)
        return kcna_fail(c, KCNA_E_ARG, "build: unknown kind");
    KCNA_TRY(bind(c));
    kcna_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof *st);
    free_state(c);
    reset_phase_stats(c);
    c->t0 = kcna_now();
    kcna_params P = *p;
    KCNA_TRY(prepare_rows(c, p, &st->bf16_rows, &st->gram_tc));
    KCNA_TRY(kcna_nndescent_run(c, &P, st));
    const uint32_t maxl = c->cap;
    if (c->n <= P.K) P.loop_i = 0; // clamping of src/kgraph.cpp:1320-1327
    float r = 0;
    KCNA_TRY(kcna_control_recall(c, maxl, &r));
    st->loop_recall[0] = r;
    st->nndescent_time = kcna_now() - c->t0;
    kcna_log(c, &P, "nndescent done: recall@MAXL %.4f t %.3f", r, st->nndescent_time);
    KCNA_TRY(kcna_graph_alloc(c, P.nsg_R + 8));
    KCNA_TRY(kcna_pools_set_radius(c, maxl)); // init_nhoods: pools grow to MAXL (:1462-1496)
    uint64_t prune_comps = 0, bridge_comps = 0;
    int loopcount = 0;
    const uint32_t iters = P.loop_i + 1;
    for (uint32_t iter = 1; iter <= iters; ++iter) {
        double a = kcna_now();
        uint64_t pc = 0;
        KCNA_TRY(kcna_link_all(c, &P, kind == KCNA_HNSW_LAYER ? KCNA_NSG : kind, &pc));
        prune_comps += pc;
        double b = kcna_now();
        KCNA_TRY(kcna_compute_ep(c, &P, (uint64_t)P.seed * 1000003ull + iter));
        double e = kcna_now();
        if (kind != KCNA_HNSW_LAYER) KCNA_TRY(kcna_tree_grow(c, &P, (uint64_t)P.seed * 7919ull + iter));
        double f = kcna_now();
        KCNA_TRY(kcna_update_nhoods(c, loopcount));
        KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "loop sync"));
        if (loopcount < KCNA_MAX_LOOPS) {
            st->prune_time[loopcount] = b - a;
            st->inter_time[loopcount] = 0;
            st->tree_grow_time[loopcount] = f - e;
            st->buildnsg_time[loopcount] = kcna_now() - a;
            st->con_time[loopcount] = kcna_now() - c->t0;
        }
        kcna_log(c, &P, "loop %u: link %.3f ep %.3f tree_grow %.3f", iter, b - a, e - b, f - e);
        loopcount++;
        if (iter == iters) break;
        double s0 = kcna_now();
        uint64_t bc = 0;
        if (P.refine == KCNA_REFINE_POOL_SEARCH)
            KCNA_TRY(kcna_pool_search_run(c, &P, maxl, loopcount, &bc));
        else
            KCNA_TRY(kcna_bridge_view(c, &P, maxl, loopcount, &bc));
        bridge_comps += bc;
        KCNA_TRY(kcna_control_recall(c, maxl, &r));
        if (loopcount - 1 < KCNA_MAX_LOOPS) st->search_time[loopcount - 1] = kcna_now() - s0;
        if (loopcount <= KCNA_MAX_LOOPS) st->loop_recall[loopcount] = r;
        kcna_log(c, &P, "P2K %d: recall@MAXL %.4f t %.3f", loopcount, r, kcna_now() - s0);
    }
    st->loops = (uint32_t)loopcount;
    st->prune_tc = kcna_prune_tc_ok(c, kind == KCNA_HNSW_LAYER ? KCNA_NSG : kind, (int)P.nsg_R,
                                    (int)std::min(P.search_K, c->cap), P.angle) ? 1u
                   : kcna_prune_fp8_ok(c, kind, (int)P.nsg_R, (int)std::min(P.search_K, c->cap)) ? 2u : 0u;
    st->prune_comps = prune_comps;
    st->bridge_comps = bridge_comps;
    KCNA_TRY(degree_stats(c, st));
    st->total_time = kcna_now() - c->t0;
    copy_phase_stats(c, st);
    return kcna_check_device_err(c, "build");
}

kcna_status kcna_get_graph(kcna_ctx *c, uint32_t *ids, uint32_t *degrees, uint32_t *ep, uint32_t *width) {
    if (!c || !c->has_graph) return kcna_fail(c, KCNA_E_STATE, "get_graph: no graph");
    KCNA_TRY(bind(c));
    if (width) *width = c->W;
    if (ep) *ep = c->ep;
    if (ids)
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(ids, c->g_ids, (size_t)c->n * c->W * 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    if (degrees)
        KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(degrees, c->g_deg, (size_t)c->n * 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    return kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "get_graph sync");
}

kcna_status kcna_pool_capacity(kcna_ctx *c, uint32_t *cap) {
    if (!c || !c->has_pools) return kcna_fail(c, KCNA_E_STATE, "no pools");
    *cap = c->cap;
    return KCNA_OK;
}

kcna_status kcna_get_pools(kcna_ctx *c, uint32_t *ids, float *dists, uint32_t *counts, uint32_t cap) {
    if (!c || !c->has_pools) return kcna_fail(c, KCNA_E_STATE, "get_pools: no pools");
    if (cap < c->cap) return kcna_fail(c, KCNA_E_ARG, "get_pools: cap below the pool capacity");
    KCNA_TRY(bind(c));
    std::vector<uint64_t> keys((size_t)c->n * c->cap);
    std::vector<uint32_t> cnt(c->n);
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(keys.data(), c->pool, keys.size() * 8, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(cnt.data(), c->pool_cnt, (size_t)c->n * 4, cudaMemcpyDeviceToHost, c->stream), "d2h"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync"));
    for (uint32_t i = 0; i < c->n; ++i) {
        uint32_t k = std::min(cnt[i], c->cap);
        if (counts) counts[i] = k;
        for (uint32_t j = 0; j < cap; ++j) {
            uint64_t key = j < k ? keys[(size_t)i * c->cap + j] : KCNA_EMPTY_KEY_H;
            if (ids) ids[(size_t)i * cap + j] = j < k ? (uint32_t)(key & 0xFFFFFFFFull) >> 2 : 0xFFFFFFFFu;
            if (dists) {
                uint32_t bits = (uint32_t)(key >> 32);
                float f;
                memcpy(&f, &bits, 4);
                dists[(size_t)i * cap + j] = j < k ? f : INFINITY;
            }
        }
    }
    return KCNA_OK;
}

kcna_status kcna_set_pools(kcna_ctx *c, const kcna_params *p, const uint32_t *ids, const float *dists,
                           const uint32_t *counts, uint32_t cap) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "set_pools: no rows");
    if (!p || !ids || !dists || !counts || cap == 0) return kcna_fail(c, KCNA_E_ARG, "set_pools: null argument");
    KCNA_TRY(bind(c));
    free_state(c);
    const uint32_t maxl = std::max(std::max(std::max(p->L, p->K), std::max(p->search_L, p->search_K)), cap);
    if (maxl > 1024) return kcna_fail(c, KCNA_E_ARG, "set_pools: capacity above 1024");
    c->cap = maxl;
    std::vector<uint64_t> keys((size_t)c->n * maxl, KCNA_EMPTY_KEY_H);
    std::vector<uint32_t> cnt(c->n);
    for (uint32_t i = 0; i < c->n; ++i) {
        uint32_t k = std::min(counts[i], cap);
        cnt[i] = k;
        for (uint32_t j = 0; j < k; ++j) {
            uint32_t id = ids[(size_t)i * cap + j];
            if (id >= c->n) return kcna_fail(c, KCNA_E_ARG, "set_pools: id out of range");
            float f = dists[(size_t)i * cap + j];
            uint32_t bits;
            memcpy(&bits, &f, 4);
            keys[(size_t)i * maxl + j] = ((uint64_t)bits << 32) | ((uint64_t)id << 2);
        }
    }
    // two spare entries: the tile prunes copy pool prefixes from an even index
    // in 16-byte units, which can reach one entry past the last row
    KCNA_TRY(kcna_alloc(c, &c->pool, keys.size() + 2, "pool"));
    KCNA_TRY(kcna_alloc(c, &c->pool_cnt, c->n, "pool_cnt"));
    KCNA_TRY(kcna_alloc(c, &c->radius, c->n, "radius"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->pool, keys.data(), keys.size() * 8, cudaMemcpyHostToDevice, c->stream), "h2d"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->pool_cnt, cnt.data(), (size_t)c->n * 4, cudaMemcpyHostToDevice, c->stream), "h2d"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync"));
    c->has_pools = true;
    return kcna_pools_set_radius(c, maxl);
}

kcna_status kcna_prune(kcna_ctx *c, const kcna_params *p, kcna_kind kind) {
    if (!c || !p) return kcna_fail(c, KCNA_E_ARG, "prune: null argument");
    KCNA_TRY(bind(c));
    uint64_t comps = 0;
    uint32_t used = 0;
    KCNA_TRY(prepare_rows(c, p, &used));
    if (kind == KCNA_CAGRA)
        KCNA_TRY(kcna_cagra_prune(c, p));
    else
        KCNA_TRY(kcna_prune_all(c, p, kind == KCNA_HNSW_LAYER ? KCNA_NSG : kind, &comps));
    return kcna_check_device_err(c, "prune");
}

kcna_status kcna_link(kcna_ctx *c, const kcna_params *p, kcna_kind kind) {
    if (!c || !p) return kcna_fail(c, KCNA_E_ARG, "link: null argument");
    KCNA_TRY(bind(c));
    uint64_t comps = 0;
    uint32_t used = 0;
    if (kind == KCNA_CAGRA) return kcna_fail(c, KCNA_E_ARG, "link: the CAGRA rank prune has no link step");
    KCNA_TRY(prepare_rows(c, p, &used));
    KCNA_TRY(kcna_link_all(c, p, kind == KCNA_HNSW_LAYER ? KCNA_NSG : kind, &comps));
    return kcna_check_device_err(c, "link");
}

kcna_status kcna_pool_search(kcna_ctx *c, const kcna_params *p, uint32_t loopcount, uint64_t *comps) {
    if (!c || !p) return kcna_fail(c, KCNA_E_ARG, "pool search: null argument");
    KCNA_TRY(bind(c));
    uint64_t cc = 0;
    KCNA_TRY(kcna_pool_search_run(c, p, c->cap, (int)loopcount, &cc));
    if (comps) *comps = cc;
    return kcna_check_device_err(c, "pool search");
}

kcna_status kcna_refine_pools(kcna_ctx *c, const kcna_params *p, uint32_t loopcount, uint64_t *comps) {
    if (!c || !p) return kcna_fail(c, KCNA_E_ARG, "refine: null argument");
    if (loopcount == 0) return kcna_fail(c, KCNA_E_ARG, "refine: loopcount must be >= 1");
    if (!c->has_pools || !c->has_graph) return kcna_fail(c, KCNA_E_STATE, "refine: needs pools and a graph");
    KCNA_TRY(bind(c));
    uint32_t used = 0;
    KCNA_TRY(prepare_rows(c, p, &used));
    KCNA_TRY(kcna_cand_alloc(c, p));
    // as kcna_build between prune loops: UpdateNhoods of the loop that built
    // this graph (loopcount - 1; 0 marks every edge new), then the refinement
    KCNA_TRY(kcna_update_nhoods(c, (int)loopcount - 1));
    uint64_t cc = 0;
    if (p->refine == KCNA_REFINE_POOL_SEARCH)
        KCNA_TRY(kcna_pool_search_run(c, p, c->cap, (int)loopcount, &cc));
    else
        KCNA_TRY(kcna_bridge_view(c, p, c->cap, (int)loopcount, &cc));
    if (comps) *comps = cc;
    return kcna_check_device_err(c, "refine");
}

kcna_status kcna_get_edge_isnew(kcna_ctx *c, uint8_t *isnew) {
    if (!c || !isnew) return kcna_fail(c, KCNA_E_ARG, "get_edge_isnew: null argument");
    if (!c->has_graph || !c->g_isnew) return kcna_fail(c, KCNA_E_STATE, "get_edge_isnew: no graph");
    KCNA_TRY(bind(c));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(isnew, c->g_isnew, (size_t)c->n * c->W, cudaMemcpyDeviceToHost,
                                                c->stream), "d2h"));
    return kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
}

kcna_status kcna_set_graph(kcna_ctx *c, const uint32_t *ids, const uint32_t *degrees, uint32_t width, uint32_t ep) {
    if (!c || !c->X) return kcna_fail(c, KCNA_E_STATE, "set_graph: no rows");
    if (!ids || !degrees || width == 0 || width > 4096 || ep >= c->n) return kcna_fail(c, KCNA_E_ARG, "set_graph: bad argument");
    KCNA_TRY(bind(c));
    for (uint32_t i = 0; i < c->n; ++i)
        if (degrees[i] > width) return kcna_fail(c, KCNA_E_ARG, "set_graph: degree above width");
    if (c->W != width) {
        c->W = 0;
        if (c->g_ids) {
            kcna_release(c, c->g_ids);
            c->g_ids = nullptr;
        }
    }
    KCNA_TRY(kcna_graph_alloc(c, width));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->g_ids, ids, (size_t)c->n * width * 4, cudaMemcpyHostToDevice, c->stream), "h2d"));
    KCNA_TRY(kcna_cuda_check(c, cudaMemcpyAsync(c->g_deg, degrees, (size_t)c->n * 4, cudaMemcpyHostToDevice, c->stream), "h2d"));
    KCNA_TRY(kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "sync"));
    c->ep = ep;
    c->has_graph = true;
    return KCNA_OK;
}

kcna_status kcna_search(kcna_ctx *c, const float *queries, uint32_t m, uint64_t q_stride, const uint32_t *init_ids,
                        uint32_t L, uint32_t k, uint32_t *out_ids, float *out_dists) {
    if (!c || !c->has_graph) return kcna_fail(c, KCNA_E_STATE, "search: no graph");
    if (!queries || !out_ids || !out_dists || m == 0 || q_stride < (uint64_t)c->d * 4)
        return kcna_fail(c, KCNA_E_ARG, "search: bad argument");
    if (L == 0 || L > std::min<uint32_t>(2048, c->n) || k == 0 || k > L)
        return kcna_fail(c, KCNA_E_ARG, "search: need 0 < k <= L <= min(2048, n)");
    KCNA_TRY(bind(c));
    std::vector<uint32_t> init;
    if (init_ids) {
        init.assign(init_ids, init_ids + (size_t)m * L);
    } else {
        // entry point, its graph neighbours, then seeded random distinct ids
        std::vector<uint32_t> row(c->W), one;
        uint32_t dg = 0;
        cudaMemcpy(row.data(), c->g_ids + (size_t)c->ep * c->W, c->W * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&dg, c->g_deg + c->ep, 4, cudaMemcpyDeviceToHost);
        std::set<uint32_t> seen;
        one.push_back(c->ep);
        seen.insert(c->ep);
        for (uint32_t j = 0; j < std::min(dg, c->W) && one.size() < L; ++j)
            if (row[j] < c->n && seen.insert(row[j]).second) one.push_back(row[j]);
        std::mt19937 rng(2024);
        while (one.size() < L) {
            uint32_t id = rng() % c->n;
            if (seen.insert(id).second) one.push_back(id);
        }
        init.resize((size_t)m * L);
        for (uint32_t i = 0; i < m; ++i) std::copy(one.begin(), one.end(), init.begin() + (size_t)i * L);
    }
    float *dq = nullptr, *od = nullptr;
    uint32_t *di = nullptr, *oid = nullptr;
    kcna_status s = to_device_rows(c, queries, m, q_stride, &dq);
    if (s == KCNA_OK) s = kcna_alloc(c, &di, init.size(), "init ids");
    if (s == KCNA_OK) s = kcna_alloc(c, &oid, (size_t)m * k, "out ids");
    if (s == KCNA_OK) s = kcna_alloc(c, &od, (size_t)m * k, "out dists");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaMemcpyAsync(di, init.data(), init.size() * 4, cudaMemcpyHostToDevice, c->stream), "h2d");
    if (s == KCNA_OK) s = kcna_search_device(c, dq, m, di, L, k, oid, od);
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_ids, oid, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK)
        s = kcna_cuda_check(c, cudaMemcpyAsync(out_dists, od, (size_t)m * k * 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    if (s == KCNA_OK) s = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "search sync");
    kcna_release(c, dq);
    kcna_release(c, di);
    kcna_release(c, oid);
    kcna_release(c, od);
    return s == KCNA_OK ? kcna_check_device_err(c, "search") : s;
}

} // extern "C"
