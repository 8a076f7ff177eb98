// ref_harness.cpp - TEST INFRASTRUCTURE, not product code.
//
// Compiles the reference's own src/kgraph.cpp, unmodified, into this
// translation unit (read from the reference tree by oracle/build_ref.sh,
// never copied into this repository) against the self-written Boost-subset
// shim in oracle/compat, and exposes its build-path functions through a small
// C interface so that tests can pin the oracle restatement
// (oracle/kcna_oracle.cpp) and generate golden fixtures from the reference
// itself.  `class` is defined to `struct` around the include only to give this
// harness access to KGraphConstructor's internals (pools, nn_nsg lists).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <malloc.h>
#include <mutex>
#include <queue>
#include <random>
#include <stack>
#include <stdexcept>
#include <unordered_set>
#include <vector>
#include <sys/resource.h>
#include <execinfo.h>
#include <signal.h>
#include <unistd.h>
#include <omp.h>
#include <boost/timer/timer.hpp>
#include <boost/progress.hpp>
#include <boost/dynamic_bitset.hpp>
#include <boost/accumulators/accumulators.hpp>
#include <boost/accumulators/statistics/stats.hpp>
#include <boost/accumulators/statistics/mean.hpp>
#include <boost/accumulators/statistics/moment.hpp>
#include <boost/smart_ptr/detail/spinlock.hpp>
#include <boost/assert.hpp>

#define class struct
#include "kgraph.cpp"
#undef class
#include "kgraph-data.h"

#include "kcna.h"

using namespace kgraph;
typedef MatrixOracle<float, metric::l2sqr> RefOracle;

namespace {

struct Quiet { // the reference prints progress to stdout; silence it in tests
    std::streambuf *old;
    Quiet() : old(std::cout.rdbuf(nullptr)) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

void fill(Matrix<float> &M, const float *X, uint64_t stride, unsigned n, unsigned d) {
    M.resize(n, d);
    M.zero();
    for (unsigned i = 0; i < n; ++i) std::memcpy(M[i], X + (uint64_t)i * stride, sizeof(float) * d);
}

KGraph::IndexParams to_params(const kcna_params *p) {
    KGraph::IndexParams q;
    q.K = p->K;
    q.L = p->L;
    q.S = p->S;
    q.R = p->R;
    q.iterations = p->iterations;
    q.controls = p->controls;
    q.seed = p->seed;
    q.nthreads = p->nthreads;
    q.delta = p->delta;
    q.recall = p->recall;
    q.nsg_R = p->nsg_R;
    q.search_L = p->search_L;
    q.search_K = p->search_K;
    q.step = p->step;
    q.massq_S = p->massq_S;
    q.loop_i = p->loop_i;
    q.tau = p->tau;
    q.angle = p->angle;
    q.prune = 0;
    q.reverse = 0;
    return q;
}

// A constructor that runs no NN-descent iteration: used to hold given pools.
KGraphConstructor *empty_constructor(RefOracle &O, const kcna_params *p, const uint32_t *pid, const float *pd,
                                     const uint32_t *pcnt, uint32_t cap) {
    KGraph::IndexParams q = to_params(p);
    q.iterations = 0;
    q.controls = 1;
    KGraph::IndexInfo info;
    KGraphConstructor *con = new KGraphConstructor(O, q, &info);
    con->init_nhoods();
    unsigned n = O.size();
    for (unsigned i = 0; i < n && pid; ++i) {
        auto &h = con->nhoods[i];
        h.pool.assign(std::max<size_t>(h.pool.size(), cap + 1), Neighbor());
        h.L = std::min<unsigned>(pcnt[i], cap);
        for (unsigned j = 0; j < h.L; ++j) {
            Neighbor nb(pid[(uint64_t)i * cap + j], pd[(uint64_t)i * cap + j], false);
            h.pool[j] = nb;
        }
    }
    return con;
}

void store_graph(KGraphConstructor *con, unsigned n, uint32_t *out_ids, float *out_d, uint32_t *out_deg,
                 uint32_t width) {
    for (unsigned i = 0; i < n; ++i) {
        auto &g = con->nhoods[i].nn_nsg;
        out_deg[i] = (uint32_t)g.size();
        for (uint32_t j = 0; j < width; ++j) {
            out_ids[(uint64_t)i * width + j] = j < g.size() ? g[j].id : 0xFFFFFFFFu;
            if (out_d) out_d[(uint64_t)i * width + j] = j < g.size() ? g[j].dist : 0.f;
        }
    }
}

} // namespace

extern "C" {

// A fault inside the reference's code (CPU) prints the stack of function names
// to stderr and ends the process with status 70 instead of dying by a signal,
// so that a run log says where it happened.
static void kref_fault_handler(int sig) {
    void *frames[64];
    const int n = backtrace(frames, 64);
    const char msg[] = "kref: fault in the reference's code, stack:\n";
    (void)!write(2, msg, sizeof msg - 1);
    backtrace_symbols_fd(frames, n, 2);
    (void)sig;
    _exit(70);
}

int kref_trap_faults(void) {
    struct sigaction sa;
    std::memset(&sa, 0, sizeof sa);
    sa.sa_handler = kref_fault_handler;
    int rc = 0;
    rc |= sigaction(SIGSEGV, &sa, nullptr);
    rc |= sigaction(SIGBUS, &sa, nullptr);
    rc |= sigaction(SIGFPE, &sa, nullptr);
    rc |= sigaction(SIGILL, &sa, nullptr);
    return rc;
}

float kref_l2(const float *a, const float *b, uint32_t d) { return metric::l2sqr::apply<float>(a, b, d); }

int kref_linear_search(const float *X, uint64_t stride, uint32_t n, uint32_t d, const uint32_t *ids, uint32_t m,
                       uint32_t k, uint32_t *out_ids, float *out_d) {
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < (int)m; ++i) {
        std::vector<Neighbor> nns;
        LinearSearch(O, ids[i], k, &nns);
        for (uint32_t j = 0; j < k; ++j) {
            out_ids[(uint64_t)i * k + j] = nns[j].id;
            out_d[(uint64_t)i * k + j] = nns[j].dist;
        }
    }
    return 0;
}

int kref_nndescent(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p, int nthreads,
                   uint32_t *pool_ids, float *pool_d, uint32_t *pool_cnt, uint32_t cap, float *iter_recall,
                   uint32_t *iters, float *final_recall) {
    Quiet quiet;
    omp_set_num_threads(nthreads);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraph::IndexParams q = to_params(p);
    KGraph::IndexInfo info;
    KGraphConstructor con(O, q, &info);
    *iters = (uint32_t)con.allrecall.size();
    for (size_t i = 0; i < con.allrecall.size() && i < KCNA_MAX_ITERS; ++i) iter_recall[i] = con.allrecall[i];
    *final_recall = con.evaluate();
    for (unsigned i = 0; i < n && pool_ids; ++i) {
        auto &h = con.nhoods[i];
        pool_cnt[i] = std::min<uint32_t>(h.L, cap);
        for (unsigned j = 0; j < cap; ++j) {
            pool_ids[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].id : 0xFFFFFFFFu;
            pool_d[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].dist : INFINITY;
        }
    }
    return 0;
}

int kref_prune(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
               const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap, uint32_t *out_ids,
               float *out_d, uint32_t *out_deg, uint32_t width) {
    Quiet quiet;
    omp_set_num_threads(1);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraphConstructor *con = empty_constructor(O, p, pid, pd, pcnt, cap);
    if (kind == KCNA_CAGRA) {
        // BuildCagra (src/kgraph.cpp:2818-2829) step by step, with one addition:
        // CagraReverse sorts each reverse list by rank only (std::sort), which
        // leaves the order of equal ranks unspecified; they are put in
        // increasing source id before CagraMerge, the order the oracle states.
        std::vector<std::vector<unsigned>> indexes(n);
        std::vector<std::vector<RankNeighbor>> regra(n);
        con->CagraComputeRoute(indexes, con->params.K / 2);
        con->CagraReverse(indexes, regra);
        for (auto &r : regra)
            std::stable_sort(r.begin(), r.end(), [](const RankNeighbor &a, const RankNeighbor &b) {
                return a.rank != b.rank ? a.rank < b.rank : a.id < b.id;
            });
        con->CagraMerge(indexes, regra);
        con->UpdateNhoods();
    }
    for (unsigned q = 0; q < n && kind != KCNA_CAGRA; ++q) {
        if (kind == KCNA_TAUMNG)
            con->taumg_sync_prune(q);
        else if (kind == KCNA_ALPHAPG)
            con->alphapg_sync_prune(q);
        else
            con->nsg_sync_prune(q);
    }
    store_graph(con, n, out_ids, out_d, out_deg, width);
    delete con;
    return 0;
}

int kref_link(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
              const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap, uint32_t *out_ids,
              float *out_d, uint32_t *out_deg, uint32_t width) {
    Quiet quiet;
    omp_set_num_threads(1);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraphConstructor *con = empty_constructor(O, p, pid, pd, pcnt, cap);
    con->pruneAgain.resize(n);
    con->pruneAgain.set();
    if (kind == KCNA_TAUMNG)
        con->taumg_Link();
    else if (kind == KCNA_ALPHAPG)
        con->alphapg_Link();
    else
        con->nsg_Link();
    store_graph(con, n, out_ids, out_d, out_deg, width);
    delete con;
    return 0;
}

// inSearch (src/kgraph.cpp:3667-3688) of loop `loopcount` on the given pools
// over the given graph; pools out (n x cap) and the scan rate it returns.
int kref_pool_search(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
                     const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap, const uint32_t *g_ids,
                     const uint32_t *g_deg, uint32_t width, uint32_t loopcount, int nthreads, uint32_t *out_ids,
                     float *out_d, uint32_t *out_cnt, float *scan) {
    Quiet quiet;
    omp_set_num_threads(nthreads);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraphConstructor *con = empty_constructor(O, p, pid, pd, pcnt, cap);
    for (unsigned i = 0; i < n; ++i) {
        con->nhoods[i].nn_nsg.clear();
        for (unsigned j = 0; j < std::min(g_deg[i], width); ++j)
            con->nhoods[i].nn_nsg.push_back(Neighbor(g_ids[(uint64_t)i * width + j], 0.f, false));
    }
    con->loopcount = loopcount;
    con->inSearch();
    *scan = con->search_cc.empty() ? 0.f : con->search_cc.back();
    for (unsigned i = 0; i < n; ++i) {
        auto &h = con->nhoods[i];
        out_cnt[i] = std::min<uint32_t>(h.L, cap);
        for (unsigned j = 0; j < cap; ++j) {
            out_ids[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].id : 0xFFFFFFFFu;
            out_d[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].dist : INFINITY;
        }
    }
    delete con;
    return 0;
}

// One P2K refinement step as buildFastNSG runs it between prune loops
// (src/kgraph.cpp:3813-3843): UpdateNhoods over the graph g (:3537-3584),
// then BridgeView (:2478-2663) with loopcount `loop`.  Pools in: ids,
// distances, counts and per-entry flags (bit 0 flag, bit 1 isnew) when
// `pflags` is given, else flag = isnew = false.  For loop 1 every edge of g is
// new; for loop >= 2 an edge is new when it is not in g_old.  Out: the pools
// with their flags, the isnew flag of every edge of g (n x width bytes) and
// the distance evaluations of the BridgeView join.
int kref_refine(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p, const uint32_t *pid,
                const float *pd, const uint32_t *pcnt, const uint8_t *pflags, uint32_t cap, const uint32_t *g_ids,
                const uint32_t *g_deg, const uint32_t *g_old, const uint32_t *g_old_deg, uint32_t width, uint32_t loop,
                int nthreads, uint32_t *out_ids, float *out_d, uint32_t *out_cnt, uint8_t *out_flags,
                uint8_t *out_isnew, uint64_t *comps) {
    Quiet quiet;
    omp_set_num_threads(nthreads);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraphConstructor *con = empty_constructor(O, p, pid, pd, pcnt, cap);
    for (unsigned i = 0; i < n; ++i) {
        auto &h = con->nhoods[i];
        for (unsigned j = 0; j < h.L && pflags; ++j) {
            h.pool[j].flag = (pflags[(uint64_t)i * cap + j] & 1) != 0;
            h.pool[j].isnew = (pflags[(uint64_t)i * cap + j] & 2) != 0;
        }
        h.old_nsg.clear();
        for (unsigned j = 0; g_old && j < std::min(g_old_deg[i], width); ++j)
            h.old_nsg.push_back(g_old[(uint64_t)i * width + j]);
        h.nn_nsg.clear();
        for (unsigned j = 0; j < std::min(g_deg[i], width); ++j)
            h.nn_nsg.push_back(Neighbor(g_ids[(uint64_t)i * width + j], 0.f, false));
    }
    con->loopcount = loop - 1; // buildFastNSG: UpdateNhoods at the end of buildNSG, then loopcount++
    con->UpdateNhoods();
    for (unsigned i = 0; i < n; ++i)
        for (uint32_t j = 0; j < width; ++j)
            out_isnew[(uint64_t)i * width + j] =
                j < con->nhoods[i].nn_nsg.size() ? (con->nhoods[i].nn_nsg[j].isnew ? 1 : 0) : 0;
    con->loopcount = loop;
    con->BridgeView();
    // the reference keeps only the scan rate cc / (n (n - 1) / 2), summed in FP32 over the rounds
    const float rate = con->search_cc.empty() ? 0.f : con->search_cc.back();
    *comps = (uint64_t)std::llround((double)rate * ((double)n * (double)(n - 1) / 2.0));
    for (unsigned i = 0; i < n; ++i) {
        auto &h = con->nhoods[i];
        out_cnt[i] = std::min<uint32_t>(h.L, cap);
        for (unsigned j = 0; j < cap; ++j) {
            out_ids[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].id : 0xFFFFFFFFu;
            out_d[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].dist : INFINITY;
            out_flags[(uint64_t)i * cap + j] =
                j < h.L ? (uint8_t)((h.pool[j].flag ? 1 : 0) | (h.pool[j].isnew ? 2 : 0)) : 0;
        }
    }
    delete con;
    return 0;
}

int kref_beam_search(const float *X, uint64_t stride, uint32_t n, uint32_t d, const uint32_t *g_ids,
                     const uint32_t *g_deg, uint32_t width, const float *Q, uint64_t qstride, uint32_t m,
                     const uint32_t *init_ids, uint32_t L, uint32_t k, uint32_t *out_ids, float *out_d) {
    Quiet quiet;
    omp_set_num_threads(1);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    kcna_params p;
    std::memset(&p, 0, sizeof p);
    p.K = p.L = p.search_K = std::max<uint32_t>(L, 2);
    p.S = 1;
    p.search_L = L;
    p.nsg_R = width;
    KGraphConstructor *con = empty_constructor(O, &p, nullptr, nullptr, nullptr, 0);
    for (unsigned i = 0; i < n; ++i) {
        con->nhoods[i].nn_nsg.clear();
        for (unsigned j = 0; j < std::min(g_deg[i], width); ++j)
            con->nhoods[i].nn_nsg.push_back(Neighbor(g_ids[(uint64_t)i * width + j], 0.f, false));
    }
    auto &seed_pool = con->nhoods[0].pool;
    if (seed_pool.size() < L + 1) seed_pool.resize(L + 1);
    for (uint32_t i = 0; i < m; ++i) {
        for (uint32_t j = 0; j < L; ++j) seed_pool[j].id = init_ids[(uint64_t)i * L + j];
        std::vector<Neighbor> pool;
        con->get_neighbors(Q + (uint64_t)i * qstride, 0, L, pool);
        for (uint32_t j = 0; j < k; ++j) {
            out_ids[(uint64_t)i * k + j] = pool[j].id;
            out_d[(uint64_t)i * k + j] = pool[j].dist;
        }
    }
    delete con;
    return 0;
}

// Full reference build through its public API (KGraph::create + buildFast*),
// writing the NSG-format index and the run CSV to the given paths.
int kref_build(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p, int nthreads,
               const char *index_path, const char *csv_path, int quiet) {
    std::streambuf *old = quiet ? std::cout.rdbuf(nullptr) : nullptr;
    omp_set_num_threads(nthreads);
    Matrix<float> M;
    fill(M, X, stride, n, d);
    RefOracle O(M);
    KGraph::IndexParams q = to_params(p);
    KGraph::IndexInfo info;
    KGraph *kg = KGraph::create();
    if (kind == KCNA_TAUMNG)
        kg->buildFastTauMNG(O, q, &info, index_path, csv_path);
    else if (kind == KCNA_ALPHAPG)
        kg->buildFastAlphaPG(O, q, &info, index_path, csv_path);
    else
        kg->buildFastNSG(O, q, &info, index_path, csv_path);
    delete kg;
    if (quiet) std::cout.rdbuf(old);
    return 0;
}

// Level assignment of hnsw_dataload (Matrix::getlevel, src/kgraph-data.h:186-222):
// data2file[n] (storage row -> file row) and points_num per level.
int kref_getlevel(uint32_t n, uint32_t M, uint32_t seed, int *data2file, int *points_num, uint32_t max_levels,
                  uint32_t *nlevels) {
    Matrix<float> m;
    std::vector<int> d2f, f2d, pn;
    m.getlevel(n, d2f, f2d, pn, M, seed);
    if (pn.size() > max_levels) return 1;
    std::copy(d2f.begin(), d2f.end(), data2file);
    std::copy(pn.begin(), pn.end(), points_num);
    *nlevels = (uint32_t)pn.size();
    return 0;
}

// Layered HNSW build through the reference's public API, orchestrated as its
// fasthnsw tool does (src/fasthnsw.cpp:204-342): rows stored in level order,
// one buildFastHNSW per level on the prefix of rows that reach it (nsg_R
// doubled at level 0), FatherSwapHNSWLayer0, then the hnswlib file.  X is in
// file order; single_level = 1 gives fastnsw (everything on level 0).
int kref_build_hnsw(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p, int nthreads,
                    int single_level, const char *path, int quiet) {
    std::streambuf *old = quiet ? std::cout.rdbuf(nullptr) : nullptr;
    omp_set_num_threads(nthreads);
    KGraph::IndexParams q = to_params(p);
    Matrix<float> lv;
    std::vector<int> labels, file2data, points_num;
    lv.getlevel(n, labels, file2data, points_num, q.nsg_R, q.seed);
    if (single_level) points_num.assign(1, (int)n);
    Matrix<float> M;
    M.resize(n, d);
    M.zero();
    for (uint32_t i = 0; i < n; ++i) std::memcpy(M[i], X + (uint64_t)labels[i] * stride, (size_t)d * 4);
    std::vector<int> levels;
    for (int l = (int)points_num.size() - 1; l >= 0; --l)
        for (int j = 0; j < points_num[l]; ++j) levels.push_back(l);
    const size_t maxM = q.nsg_R, maxM0 = 2 * (size_t)q.nsg_R, Mlinks = q.nsg_R;
    const size_t links = maxM * 4 + 4, links0 = maxM0 * 4 + 4;
    const size_t per = links0 + 4 * (size_t)d + 8, label_off = links0 + 4 * (size_t)d, data_off = links0;
    std::vector<char *> ll(n, nullptr);
    for (uint32_t i = 0; i < n && levels[i] > 0; ++i) ll[i] = (char *)calloc(links * levels[i] + 1, 1);
    RefOracle O(M);
    KGraph *kg = KGraph::create();
    KGraph::IndexInfo info;
    unsigned ep = 0, layer_ep = 0, size = 0;
    char *level0 = nullptr;
    for (int level = (int)points_num.size() - 1; level >= 0; --level) {
        size += points_num[level];
        O.set_size(size);
        if (size == 1 && level > 0) {
            std::memset(ll[0] + (size_t)(level - 1) * links, 0, 2);
            if (level == (int)points_num.size() - 1) ep = 0;
            continue;
        }
        if (level > 0) {
            kg->buildFastHNSW(O, q, &info, "", "", level0, ll.data(), (unsigned)level, &layer_ep);
        } else {
            q.nsg_R *= 2;
            kg->buildFastHNSW(O, q, &info, "", "", level0, ll.data(), 0, &layer_ep, per);
            level0 = (char *)calloc((size_t)n * per, 1);
            kg->FatherSwapHNSWLayer0(O, q, level0);
        }
        if (level == (int)points_num.size() - 1) ep = layer_ep;
    }
    delete kg;
    for (uint32_t i = 0; i < n; ++i) {
        const size_t label = (size_t)labels[i];
        std::memcpy(level0 + (size_t)i * per + data_off, M[i], (size_t)d * 4);
        std::memcpy(level0 + (size_t)i * per + label_off, &label, sizeof label);
    }
    std::ofstream out(path, std::ios::binary);
    const size_t zero = 0, nn = n, efc = q.search_K;
    const int maxlevel = levels.empty() ? 0 : levels[0];
    const double mult = 1 / std::log(1.0 * Mlinks);
    out.write((const char *)&zero, 8);
    out.write((const char *)&nn, 8);
    out.write((const char *)&nn, 8);
    out.write((const char *)&per, 8);
    out.write((const char *)&label_off, 8);
    out.write((const char *)&data_off, 8);
    out.write((const char *)&maxlevel, 4);
    out.write((const char *)&ep, 4);
    out.write((const char *)&maxM, 8);
    out.write((const char *)&maxM0, 8);
    out.write((const char *)&Mlinks, 8);
    out.write((const char *)&mult, 8);
    out.write((const char *)&efc, 8);
    out.write(level0, (std::streamsize)((size_t)n * per));
    for (uint32_t i = 0; i < n; ++i) {
        const unsigned sz = levels[i] > 0 ? (unsigned)(links * levels[i]) : 0u;
        out.write((const char *)&sz, 4);
        if (sz) out.write(ll[i], sz);
    }
    free(level0);
    for (char *x : ll) free(x);
    if (quiet) std::cout.rdbuf(old);
    return out ? 0 : 1;
}

} // extern "C"
