// kcna_oracle.cpp - TEST INFRASTRUCTURE, not product code.
//
// CPU restatement of FastKCNA's graph-construction path (NN-descent, occlusion
// prune + link, entry point, tree_grow, UpdateNhoods, P2K "BridgeView", the
// CAGRA-style rank prune) written
// from the reference's behaviour, function by function, each citing the
// reference file:line it follows (paths relative to the reference project).
// It is the checker for the CUDA library: the tests, the smoke check and the
// bench's CPU-baseline leg are the only callers.  Nothing in the product links it.
//
// One deliberate difference from the reference: the squared L2 distance is the
// library's canonical FP32 form, a single sequential fused multiply-add chain
// over the dimensions (acc = fma(x-y, x-y, acc), k = 0..d-1), so that the CUDA
// kernels and this oracle agree bit for bit on float data.  The reference sums
// in a SIMD lane order on x86 (src/metric.cpp:45-78) and in a plain scalar loop
// elsewhere (src/kgraph-data.h:51-60); on integer-valued data every order gives
// the same exact value.  The oracle is pinned against the reference itself
// (compiled from its own sources by oracle/build_ref.sh) by the golden fixtures
// under tests/golden/.
//
// Two more points where the reference is ill-defined and this file states a
// choice:
//  * findroot (src/kgraph.cpp:2203-2214) declares an inner `id` initialised from
//    itself (undefined behaviour).  The reference's builds evaluate that read
//    as 0 (with -ftrivial-auto-var-init=zero, and likewise with plain -O3 on
//    x86-64: the links between C2 clusters then start in node 0's cluster),
//    so node 0's pool is scanned here too.
//  * InterInsert (src/kgraph.cpp:2051-2084) runs under OpenMP with the order
//    of appended reverse edges set by thread timing; here (and on the GPU) the
//    reverse edges of a node are appended in increasing source id, and the
//    re-prune sorts stably by distance, so results are deterministic.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <random>
#include <stack>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "kcna.h"

namespace kcnao {

static const double kPi = 3.14159265358979323846264;

// Pool entry, the reference's Neighbor (src/neighbor.h:25-43).
struct Nb {
    uint32_t id;
    float dist;
    bool flag;   // newly found, not yet used in a join
    bool isnew;  // new relative to the previous prune loop
    int16_t pid; // index of the kept neighbour that occluded this entry
    Nb() : id(0), dist(std::numeric_limits<float>::max()), flag(false), isnew(true), pid(-1) {}
    Nb(uint32_t i, float d, bool f) : id(i), dist(d), flag(f), isnew(true), pid(-1) {}
};
static inline bool operator<(const Nb &a, const Nb &b) { return a.dist < b.dist; }

// Canonical FP32 squared L2: one fused multiply-add chain in dimension order.
static inline float l2(const float *a, const float *b, unsigned d) {
    float acc = 0.0f;
    for (unsigned k = 0; k < d; ++k) {
        float t = a[k] - b[k];
        acc = std::fma(t, t, acc);
    }
    return acc;
}

struct Data {
    const float *X;
    uint64_t stride; // floats per row
    unsigned n;      // rows visible (IndexOracle::size after set_size)
    unsigned d;
    const float *row(unsigned i) const { return X + (uint64_t)i * stride; }
    float operator()(unsigned i, unsigned j) const { return l2(row(i), row(j), d); }
    float q(const float *query, unsigned i) const { return l2(query, row(i), d); }
};

// Sorted insert with duplicate check; src/kgraph.cpp:261-298 (InsertIntoPool).
// addr[0..K-1] sorted ascending, addr[K] receives the overflow.  Returns the
// insert position, K+1 on a duplicate id among equal distances.
static inline int insert_into_pool(Nb *addr, unsigned K, Nb nn) {
    int left = 0, right = (int)K - 1;
    if (addr[left].dist > nn.dist) {
        memmove((char *)&addr[left + 1], &addr[left], K * sizeof(Nb));
        addr[left] = nn;
        return left;
    }
    if (addr[right].dist < nn.dist) {
        addr[K] = nn;
        return (int)K;
    }
    while (left < right - 1) {
        int mid = (left + right) / 2;
        if (addr[mid].dist > nn.dist)
            right = mid;
        else
            left = mid;
    }
    while (left > 0) {
        if (addr[left].dist < nn.dist) break;
        if (addr[left].id == nn.id) return (int)K + 1;
        left--;
    }
    if (addr[left].id == nn.id || addr[right].id == nn.id) return (int)K + 1;
    memmove((char *)&addr[right + 1], &addr[right], (K - right) * sizeof(Nb));
    addr[right] = nn;
    return right;
}

// Insert keeping the K+1-slot list sorted with ties placed after equals;
// src/kgraph.cpp:227-260 (UpdateKnnListHelper).
static inline unsigned update_knn_list(Nb *addr, unsigned K, Nb nn) {
    unsigned i = K, j;
    while (i > 0) {
        j = i - 1;
        if (addr[j].dist <= nn.dist) break;
        i = j;
    }
    unsigned l = i;
    while (l > 0) {
        j = l - 1;
        if (addr[j].dist < nn.dist) break;
        if (addr[j].id == nn.id) return K + 1;
        l = j;
    }
    j = K;
    while (j > i) {
        addr[j] = addr[j - 1];
        --j;
    }
    addr[i] = nn;
    return i;
}

// size distinct pseudo-random ids < N; src/kgraph.cpp:82-110 (GenRandom).
template <typename RNG>
static void gen_random(RNG &rng, unsigned *addr, unsigned size, unsigned N) {
    if (N == size) {
        for (unsigned i = 0; i < size; ++i) addr[i] = i;
        return;
    }
    for (unsigned i = 0; i < size; ++i) addr[i] = rng() % (N - size);
    std::sort(addr, addr + size);
    for (unsigned i = 1; i < size; ++i)
        if (addr[i] <= addr[i - 1]) addr[i] = addr[i - 1] + 1;
    unsigned off = rng() % N;
    for (unsigned i = 0; i < size; ++i) addr[i] = (addr[i] + off) % N;
}

// Exact K-NN of base row i, self excluded, ties to the lower id;
// src/kgraph.cpp:309-330 (LinearSearch).
static void linear_search(const Data &D, unsigned i, unsigned K, std::vector<Nb> &out) {
    std::vector<Nb> nns(K + 1);
    unsigned k = 0;
    for (unsigned id = 0; id < D.n; ++id) {
        if (id == i) continue;
        Nb nn(id, D(i, id), true);
        update_knn_list(&nns[0], k, nn);
        if (k < K) ++k;
    }
    nns.resize(K);
    out.swap(nns);
}

struct Spin {
    std::atomic_flag f = ATOMIC_FLAG_INIT;
    void lock() { while (f.test_and_set(std::memory_order_acquire)) {} }
    void unlock() { f.clear(std::memory_order_release); }
};

struct Nhood { // src/kgraph.cpp:929-988
    float radius = std::numeric_limits<float>::max();
    float radiusM = 0;
    unsigned L = 0, M = 0;
    bool found = false;
    std::vector<Nb> pool;
    std::vector<Nb> nn_nsg;
    std::vector<unsigned> nn_old, nn_new, rnn_old, rnn_new, old_nsg;
    std::vector<bool> rnn_new_flag;
    Spin lock;
    Nhood() {}
    Nhood(const Nhood &) {}
    // src/kgraph.cpp:948-967 (Nhood::parallel_try_insert)
    unsigned try_insert(unsigned id, float dist) {
        if (dist > radius) return (unsigned)pool.size();
        lock.lock();
        unsigned l = (unsigned)insert_into_pool(&pool[0], L, Nb(id, dist, true));
        if (l <= L) {
            if (L + 1 < pool.size())
                ++L;
            else
                radius = pool[L - 1].dist;
        }
        lock.unlock();
        return l;
    }
};

struct Control {
    unsigned id;
    std::vector<Nb> nbrs;
};

// control recall: src/kgraph.cpp:113-169 (EvaluateRecall, the live loop :158-168)
static float evaluate_recall(const std::vector<Nb> &pool, unsigned K0, const std::vector<Nb> &knn, unsigned K) {
    if (knn.empty()) return 1.0f;
    unsigned found = 0;
    for (unsigned i = 0; i < std::min(K0, K); i++) {
        unsigned id = pool[i].id;
        for (unsigned j = 0; j < K; j++)
            if (id == knn[j].id) {
                found++;
                break;
            }
    }
    return float(found) / K;
}

// src/kgraph.cpp:194-206 (EvaluateDelta)
static float evaluate_delta(const std::vector<Nb> &pool, unsigned L, unsigned K) {
    unsigned c = 0, N = K;
    if (L < N) N = L; // entries beyond L are empty slots
    for (unsigned i = 0; i < N; ++i)
        if (pool[i].flag) ++c;
    return float(c) / K;
}

static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Builder {
    Data D;
    kcna_params P;
    int kind;
    unsigned MAXL = 0;
    unsigned ep = 0;
    unsigned width = 0;
    unsigned loopcount = 0;
    std::vector<Nhood> nh;
    std::vector<Control> controls;
    std::vector<uint8_t> pruneAgain;
    uint64_t n_comps = 0, prune_comps = 0, bridge_comps = 0;
    kcna_stats *st;
    double t0;
    bool use_prune2 = true;

    Builder(const Data &d, const kcna_params &p, int k, kcna_stats *s) : D(d), P(p), kind(k), st(s) {}

    // Parameter clamping, src/kgraph.cpp:1289-1334.
    void clamp() {
        unsigned N = D.n;
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
        MAXL = std::max(std::max(P.L, P.K), std::max(P.search_L, P.search_K));
    }

    // src/kgraph.cpp:363-387 (GenerateControl).  The reference shuffles with
    // the C library rand(); the same call sequence is reproduced with srand(1).
    void generate_controls() {
        std::vector<unsigned> index(D.n);
        for (unsigned i = 0; i < D.n; ++i) index[i] = i;
        std::srand(1);
        // libstdc++ random_shuffle: swap i with rand() % (i+1)
        for (size_t i = 1; i < index.size(); ++i) {
            size_t j = (size_t)std::rand() % (i + 1);
            std::swap(index[i], index[j]);
        }
        controls.resize(P.controls);
#pragma omp parallel for
        for (int c = 0; c < (int)P.controls; ++c) {
            controls[c].id = index[c];
            linear_search(D, index[c], MAXL, controls[c].nbrs);
        }
    }

    // src/kgraph.cpp:1001-1044 (init)
    void init() {
        unsigned N = D.n;
        for (auto &h : nh) {
            h.nn_new.resize(P.S * 2);
            h.pool.resize(P.L + 1);
            h.radius = std::numeric_limits<float>::max();
        }
#pragma omp parallel
        {
#ifdef _OPENMP
            std::mt19937 rng(P.seed ^ omp_get_thread_num());
#else
            std::mt19937 rng(P.seed);
#endif
            std::vector<unsigned> random(P.S + 1);
#pragma omp for
            for (int n = 0; n < (int)N; ++n) {
                auto &h = nh[n];
                gen_random(rng, &h.nn_new[0], (unsigned)h.nn_new.size(), N);
                gen_random(rng, &random[0], (unsigned)random.size(), N);
                h.L = P.S;
                h.M = P.S;
                unsigned i = 0;
                for (unsigned l = 0; l < h.L; ++l) {
                    if (random[i] == (unsigned)n) ++i;
                    auto &nn = h.pool[l];
                    nn.id = random[i++];
                    nn.dist = D(nn.id, n);
                    nn.flag = true;
                }
                std::sort(h.pool.begin(), h.pool.begin() + h.L);
            }
        }
    }

    // src/kgraph.cpp:1097-1117 (join) and :970-987 (Nhood::join)
    void join() {
        uint64_t cc = 0;
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : cc)
        for (int n = 0; n < (int)D.n; ++n) {
            size_t uu = 0;
            auto &h = nh[n];
            h.found = false;
            auto cb = [&](unsigned i, unsigned j) {
                float dist = D(i, j);
                ++cc;
                unsigned r = nh[i].try_insert(j, dist);
                if (r < P.K) ++uu;
                r = nh[j].try_insert(i, dist);
                if (r < P.K) ++uu;
            };
            for (unsigned i : h.nn_new) {
                for (unsigned j : h.nn_new)
                    if (i < j) cb(i, j);
                for (unsigned j : h.nn_old) cb(i, j);
            }
            h.found = uu > 0;
        }
        n_comps += cc;
    }

    // src/kgraph.cpp:1118-1202 (update)
    void update() {
        unsigned N = D.n;
        for (auto &h : nh) {
            h.nn_new.clear();
            h.nn_old.clear();
            h.rnn_new.clear();
            h.rnn_old.clear();
            h.radius = h.pool.back().dist;
        }
#pragma omp parallel for
        for (int n = 0; n < (int)N; ++n) {
            auto &h = nh[n];
            if (h.found) {
                unsigned maxl = std::min(h.M + P.S, h.L);
                unsigned c = 0, l = 0;
                while (l < maxl && c < P.S) {
                    if (h.pool[l].flag) ++c;
                    ++l;
                }
                h.M = l;
            }
            if (h.M == 0) h.M = 1; // the reference aborts here (BOOST_VERIFY, :1148)
            h.radiusM = h.pool[h.M - 1].dist;
        }
#pragma omp parallel for
        for (int n = 0; n < (int)N; ++n) {
            auto &h = nh[n];
            for (unsigned l = 0; l < h.M; ++l) {
                auto &nn = h.pool[l];
                auto &o = nh[nn.id];
                if (nn.flag) {
                    h.nn_new.push_back(nn.id);
                    if (nn.dist > o.radiusM) {
                        o.lock.lock();
                        o.rnn_new.push_back(n);
                        o.lock.unlock();
                    }
                    nn.flag = false;
                } else {
                    h.nn_old.push_back(nn.id);
                    if (nn.dist > o.radiusM) {
                        o.lock.lock();
                        o.rnn_old.push_back(n);
                        o.lock.unlock();
                    }
                }
            }
        }
        for (unsigned i = 0; i < N; ++i) {
            auto &h = nh[i];
            if (P.R && h.rnn_new.size() > P.R) {
                // reverse lists in the reference are filled in thread order and
                // shuffled; sort first so that one thread gives one result.
                std::sort(h.rnn_new.begin(), h.rnn_new.end());
                shuffle(h.rnn_new);
                h.rnn_new.resize(P.R);
            }
            h.nn_new.insert(h.nn_new.end(), h.rnn_new.begin(), h.rnn_new.end());
            if (P.R && h.rnn_old.size() > P.R) {
                std::sort(h.rnn_old.begin(), h.rnn_old.end());
                shuffle(h.rnn_old);
                h.rnn_old.resize(P.R);
            }
            h.nn_old.insert(h.nn_old.end(), h.rnn_old.begin(), h.rnn_old.end());
        }
    }
    static void shuffle(std::vector<unsigned> &v) { // libstdc++ random_shuffle over rand()
        for (size_t i = 1; i < v.size(); ++i) {
            size_t j = (size_t)std::rand() % (i + 1);
            std::swap(v[i], v[j]);
        }
    }

    // Constructor loop, src/kgraph.cpp:1281-1459.
    void nndescent() {
        t0 = now();
        clamp();
        nh.clear();
        nh.resize(D.n);
        generate_controls();
        init();
        float total = D.n * float(D.n - 1) / 2;
        unsigned it = 0;
        st->stop_condition = 0;
        st->maxl = MAXL;
        for (it = 0; it < P.iterations; ++it) {
            join();
            float dsum = 0, rsum = 0;
            for (auto const &h : nh) dsum += evaluate_delta(h.pool, h.L, P.K);
            for (auto const &c : controls) rsum += evaluate_recall(nh[c.id].pool, nh[c.id].L, c.nbrs, P.K);
            float delta = dsum / (float)nh.size();
            float recall = controls.empty() ? 0.f : rsum / (float)controls.size();
            if (it < KCNA_MAX_ITERS) {
                st->iter_delta[it] = delta;
                st->iter_recall[it] = recall;
                st->iter_time[it] = now() - t0;
            }
            st->iterations = it + 1;
            if (P.verbosity)
                fprintf(stderr, "[oracle] iteration %u recall %.4f delta %.4f cost %.6f t %.2f\n", it + 1, recall,
                        delta, n_comps / total, now() - t0);
            if (delta <= P.delta) {
                st->stop_condition = 1;
                break;
            }
            if (recall >= P.recall) {
                st->stop_condition = 2;
                break;
            }
            if (it + 1 >= P.iterations) break;
            update();
        }
        st->n_comps = n_comps;
    }

    // src/kgraph.cpp:3701-3717 (evaluate): control recall@MAXL.
    float evaluate() {
        double r = 0;
        for (auto &c : controls) r += evaluate_recall(nh[c.id].pool, nh[c.id].L, c.nbrs, MAXL);
        return controls.empty() ? 0.f : float(r / controls.size());
    }

    // src/kgraph.cpp:1462-1496 (init_nhoods)
    void init_nhoods() {
        for (auto &h : nh) {
            std::vector<unsigned>().swap(h.nn_new);
            std::vector<unsigned>().swap(h.nn_old);
            std::vector<unsigned>().swap(h.rnn_new);
            std::vector<unsigned>().swap(h.rnn_old);
            h.pool.resize(MAXL + 1);
        }
    }

    // Occlusion test of the three prune kinds:
    //   RNG   src/kgraph.cpp:1834     djk < p.dist
    //   tau   src/kgraph.cpp:2859     djk < p.dist - 3*tau
    //   angle src/kgraph.cpp:3184-86  djk < p.dist && cos_ij < cos(angle)
    bool occludes(const Nb &t, float djk, const Nb &p, float thr) const {
        if (kind == KCNA_TAUMNG) return djk < p.dist - 3 * P.tau;
        if (kind == KCNA_ALPHAPG) {
            float cos_ij = (t.dist + djk - p.dist) / 2 / std::sqrt(t.dist * djk);
            return djk < p.dist && cos_ij < thr;
        }
        return djk < p.dist;
    }
    float angle_threshold() const { return (float)std::cos(P.angle / 180 * kPi); }

    // src/kgraph.cpp:1809-1851 (nsg_sync_prune); tau :2833-2876; angle :3157-3203
    uint64_t sync_prune(unsigned q) {
        unsigned range = P.nsg_R, maxc = P.search_K;
        float thr = angle_threshold();
        width = range;
        uint64_t cc = 0;
        unsigned start = 0;
        auto &h = nh[q];
        h.nn_nsg.clear();
        if (h.pool[start].id == q) start++;
        h.nn_nsg.push_back(h.pool[start]);
        while (h.nn_nsg.size() < range && (++start) < h.L && start < maxc) {
            auto &p = h.pool[start];
            if (p.id >= D.n) continue;
            bool occ = false;
            for (unsigned t = 0; t < h.nn_nsg.size(); t++) {
                if (p.id == h.nn_nsg[t].id) {
                    occ = true;
                    break;
                }
                cc++;
                float djk = D(h.nn_nsg[t].id, p.id);
                if (occludes(h.nn_nsg[t], djk, p, thr)) {
                    occ = true;
                    p.pid = (int16_t)t;
                    break;
                }
            }
            if (!occ) h.nn_nsg.push_back(p);
        }
        for (auto &e : h.nn_nsg) e.flag = false;
        return cc;
    }

    // src/kgraph.cpp:1853-2010 (nsg_sync_prune2): incremental re-prune reusing
    // the previous loop's decisions through isnew / pid.
    uint64_t sync_prune2(unsigned q) {
        unsigned range = P.nsg_R, maxc = P.search_K;
        float thr = angle_threshold();
        width = range;
        uint64_t cc = 0;
        unsigned start = 0;
        auto &h = nh[q];
        std::vector<unsigned> temp;
        for (auto &e : h.nn_nsg)
            if (!e.flag) temp.push_back(e.id);
        auto in_temp = [&](unsigned id) { return std::find(temp.begin(), temp.end(), id) != temp.end(); };
        h.nn_nsg.clear();
        if (h.pool[start].id == q) start++;
        h.nn_nsg.push_back(h.pool[start]);
        h.nn_nsg.back().isnew = !in_temp(h.nn_nsg.back().id);
        auto full_check = [&](Nb &p, bool all) -> bool {
            for (unsigned t = 0; t < h.nn_nsg.size(); t++) {
                if (p.id == h.nn_nsg[t].id) return true;
                if (!all && !h.nn_nsg[t].isnew) continue;
                cc++;
                float djk = D(h.nn_nsg[t].id, p.id);
                if (occludes(h.nn_nsg[t], djk, p, thr)) {
                    p.pid = (int16_t)t;
                    return true;
                }
            }
            return false;
        };
        while (h.nn_nsg.size() < range && (++start) < h.L && start < maxc) {
            auto &p = h.pool[start];
            if (p.id >= D.n) continue;
            if (p.isnew) {
                if (!full_check(p, true)) {
                    h.nn_nsg.push_back(p);
                    h.nn_nsg.back().isnew = true;
                }
                continue;
            }
            bool inT = in_temp(p.id);
            if (!inT && p.pid >= 0 && (size_t)p.pid < temp.size()) {
                unsigned prune_p = temp[p.pid];
                size_t pos = 0;
                for (; pos < h.nn_nsg.size(); ++pos)
                    if (h.nn_nsg[pos].id == prune_p) break;
                if (pos < h.nn_nsg.size()) {
                    p.pid = (int16_t)pos;
                    continue;
                }
                if (!full_check(p, true)) {
                    h.nn_nsg.push_back(p);
                    h.nn_nsg.back().isnew = true;
                }
            } else if (!inT) {
                if (!full_check(p, true)) {
                    h.nn_nsg.push_back(p);
                    h.nn_nsg.back().isnew = true;
                }
            } else {
                if (!full_check(p, false)) {
                    h.nn_nsg.push_back(p);
                    h.nn_nsg.back().isnew = false;
                }
            }
        }
        for (auto &e : h.nn_nsg) e.flag = false;
        return cc;
    }

    // src/kgraph.cpp:2012-2048 (nsg_reversed_prune); tau :3038-3083; angle :3374-3422.
    // Stable sort: see the header comment.
    void reversed_prune(unsigned q) {
        unsigned range = P.nsg_R;
        float thr = angle_threshold();
        unsigned start = 0;
        auto &h = nh[q];
        std::vector<Nb> tp = h.nn_nsg;
        std::stable_sort(tp.begin(), tp.end());
        h.nn_nsg.clear();
        if (tp[start].id == q) start++;
        h.nn_nsg.push_back(tp[start]);
        while (h.nn_nsg.size() < range && (++start) < tp.size()) {
            auto &p = tp[start];
            bool occ = false;
            for (unsigned t = 0; t < h.nn_nsg.size(); t++) {
                if (p.id == h.nn_nsg[t].id) {
                    occ = true;
                    break;
                }
                float djk = D(h.nn_nsg[t].id, p.id);
                if (occludes(h.nn_nsg[t], djk, p, thr)) {
                    occ = true;
                    break;
                }
            }
            if (!occ) h.nn_nsg.push_back(p);
        }
    }

    // src/kgraph.cpp:2051-2084 (InterInsert) in deterministic form: for each
    // node des, the sources n with des in nn_nsg(n) and n not in nn_nsg(des)
    // are appended in increasing n.
    void inter_insert() {
        unsigned N = D.n;
        std::vector<std::vector<unsigned>> rev(N);
        std::vector<size_t> sz(N);
        for (unsigned n = 0; n < N; ++n) sz[n] = nh[n].nn_nsg.size();
        for (unsigned n = 0; n < N; ++n)
            for (size_t i = 0; i < sz[n]; ++i) {
                unsigned des = nh[n].nn_nsg[i].id;
                if (des >= N) continue;
                rev[des].push_back(n);
            }
#pragma omp parallel for schedule(dynamic, 100)
        for (int des = 0; des < (int)N; ++des) {
            auto &h = nh[des];
            for (unsigned n : rev[des]) {
                bool dup = false;
                for (size_t j = 0; j < sz[des]; ++j)
                    if (h.nn_nsg[j].id == n) {
                        dup = true;
                        break;
                    }
                if (dup) continue;
                h.nn_nsg.push_back(Nb(n, D(n, des), true));
            }
        }
    }

    // src/kgraph.cpp:2087-2143 (nsg_Link); taumg_Link :3085-3141; alphapg_Link :3424-3480
    void link() {
        unsigned N = D.n;
        double a = now();
        uint64_t cc = 0;
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : cc)
        for (int n = 0; n < (int)N; ++n) cc += (pruneAgain[n] || !use_prune2) ? sync_prune(n) : sync_prune2(n);
        prune_comps += cc;
        double b = now();
        inter_insert();
        std::fill(pruneAgain.begin(), pruneAgain.end(), 0);
#pragma omp parallel for schedule(dynamic, 100)
        for (int n = 0; n < (int)N; ++n)
            if (nh[n].nn_nsg.size() > P.nsg_R) {
                pruneAgain[n] = 1;
                reversed_prune(n);
            }
        double c = now();
        if (loopcount < KCNA_MAX_LOOPS) {
            st->prune_time[loopcount] = b - a;
            st->inter_time[loopcount] = c - b;
        }
    }

    // Beam search from a query; src/kgraph.cpp:1560-1623 (get_neighbors).
    // init_ids has Lw entries, already chosen by the caller.
    void beam_search(const float *query, const std::vector<unsigned> &init_ids, unsigned Lw,
                     std::vector<Nb> &pool) const {
        unsigned nd = D.n;
        pool.assign(Lw + 1, Nb());
        std::vector<uint8_t> flags(nd, 0);
        for (unsigned id : init_ids)
            if (id < nd) flags[id] = 1;
        unsigned L = 0;
        for (unsigned i = 0; i < init_ids.size(); i++) {
            unsigned id = init_ids[i];
            if (id >= nd) continue;
            pool[i] = Nb(id, D.q(query, id), true);
            L++;
        }
        std::sort(pool.begin(), pool.begin() + L);
        int k = 0;
        while (k < (int)L) {
            int nk = L;
            if (pool[k].flag) {
                pool[k].flag = false;
                unsigned n = pool[k].id;
                for (size_t m = 0; m < nh[n].nn_nsg.size(); ++m) {
                    unsigned id = nh[n].nn_nsg[m].id;
                    if (id >= nd || flags[id]) continue;
                    flags[id] = 1;
                    float dist = D.q(query, id);
                    if (dist >= pool[L - 1].dist) continue;
                    int r = insert_into_pool(pool.data(), L, Nb(id, dist, true));
                    if (L + 1 < pool.size()) ++L;
                    if (r < nk) nk = r;
                }
            }
            if (nk <= k)
                k = nk;
            else
                ++k;
        }
    }

    // src/kgraph.cpp:1528-1536 (ComputeEp) with Calcenter (src/kgraph-data.h:413-428).
    // The centroid is accumulated in double and the start node drawn from rng.
    void compute_ep(std::mt19937 &rng) {
        unsigned nd = D.n;
        std::vector<double> c(D.d, 0.0);
        for (unsigned i = 0; i < nd; ++i)
            for (unsigned j = 0; j < D.d; ++j) c[j] += D.row(i)[j];
        std::vector<float> center(D.d);
        for (unsigned j = 0; j < D.d; ++j) center[j] = (float)(c[j] / nd);
        unsigned init_point = rng() % nd;
        unsigned Lw = P.search_L;
        std::vector<unsigned> init_ids;
        std::vector<uint8_t> seen(nd, 0);
        auto &ip = nh[init_point];
        for (unsigned i = 0; i < Lw && i < ip.L; ++i) {
            init_ids.push_back(ip.pool[i].id);
            seen[ip.pool[i].id] = 1;
        }
        while (init_ids.size() < Lw) {
            unsigned id = rng() % nd;
            if (seen[id]) continue;
            seen[id] = 1;
            init_ids.push_back(id);
        }
        std::vector<Nb> pool;
        beam_search(center.data(), init_ids, Lw, pool);
        ep = pool[0].id;
    }

    // src/kgraph.cpp:2238-2270 (DFS)
    void dfs(std::vector<uint8_t> &flag, unsigned root, unsigned &cnt) {
        unsigned nd = D.n, tmp = root;
        std::stack<unsigned> s;
        s.push(root);
        if (!flag[root]) cnt++;
        flag[root] = 1;
        while (!s.empty()) {
            unsigned next = nd + 1;
            for (auto &e : nh[tmp].nn_nsg)
                if (e.id < nd && !flag[e.id]) {
                    next = e.id;
                    break;
                }
            if (next == nd + 1) {
                s.pop();
                if (s.empty()) break;
                tmp = s.top();
                continue;
            }
            tmp = next;
            flag[tmp] = 1;
            s.push(tmp);
            cnt++;
        }
    }

    // src/kgraph.cpp:2174-2236 (findroot): node 0's pool is scanned over the
    // unreached node's pool length (the self-initialised `id` read as 0).
    void findroot(std::vector<uint8_t> &flag, unsigned &root, unsigned &start, std::mt19937 &rng) {
        unsigned nd = D.n, id = nd;
        for (unsigned i = start; i < nd; i++)
            if (!flag[i]) {
                id = i;
                start = i;
                break;
            }
        if (id == nd) return;
        bool found = false;
        for (unsigned i = 0; i < nh[id].L; i++) {
            if (i >= nh[0].pool.size()) break;
            unsigned cand = nh[0].pool[i].id;
            if (cand < nd && flag[cand] && nh[cand].nn_nsg.size() < P.nsg_R) {
                root = cand;
                found = true;
                break;
            }
        }
        if (!found) {
            unsigned cnt = 0;
            while (true) {
                cnt++;
                unsigned factor = cnt / nd + 1;
                unsigned rid = rng() % nd;
                if (flag[rid] && nh[rid].nn_nsg.size() < P.nsg_R * factor) {
                    root = rid;
                    break;
                }
            }
        }
        nh[root].nn_nsg.push_back(Nb(id, D(root, id), true));
    }

    // src/kgraph.cpp:2145-2172 (tree_grow)
    void tree_grow(std::mt19937 &rng) {
        unsigned nd = D.n, root = ep, cnt = 0, start = 0;
        std::vector<uint8_t> flags(nd, 0);
        while (cnt < nd) {
            dfs(flags, root, cnt);
            if (cnt >= nd) break;
            findroot(flags, root, start, rng);
        }
        for (unsigned i = 0; i < nd; ++i)
            if (nh[i].nn_nsg.size() > width) width = (unsigned)nh[i].nn_nsg.size();
    }

    // CAGRA-style rank prune, src/kgraph.cpp:2818-2829 (BuildCagra; none of the
    // reference's build functions calls it).  With Ki = min(K, pool count):
    //  * route[j] counts the detours i -> pool[k] -> pool[j]: k < j, and
    //    pool[j] at rank l < j in pool[k]'s own list (CagraComputeRoute
    //    :2665-2757, the live loop :2707-2725);
    //  * the prune_K = K / 2 entries with the fewest detours are kept, equal
    //    counts in rank order (sort_indexes :62-76);
    //  * every kept edge i -> w gives w a reverse entry (i, its rank in i's kept
    //    list), taken by increasing rank, equal ranks by increasing source id
    //    (CagraReverse :2759-2788 sorts by rank only, so the order of equal
    //    ranks is unspecified there);
    //  * the graph alternates kept and reverse entries until prune_K are
    //    placed, one more when the last step places both (CagraMerge
    //    :2790-2816); reverse entries carry d(i, source).
    // Entries past a pool's count are absent (the reference reads them as is).
    void build_cagra() {
        const unsigned n = D.n, K = P.K, PK = K / 2;
        std::vector<std::vector<unsigned>> keep(n);
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < (int)n; ++i) {
            const auto &pool = nh[i].pool;
            const unsigned Ki = std::min(K, nh[i].L);
            std::vector<unsigned> route(Ki, 0);
            for (unsigned k = 0; k < Ki; ++k) {
                const unsigned one = pool[k].id;
                const unsigned Kl = std::min(K, nh[one].L);
                for (unsigned l = 0; l < Kl; ++l) {
                    const unsigned two = nh[one].pool[l].id;
                    for (unsigned j = std::max(k, l) + 1; j < Ki; ++j)
                        if (two == pool[j].id) {
                            ++route[j];
                            break;
                        }
                }
            }
            std::vector<unsigned> idx(Ki);
            for (unsigned j = 0; j < Ki; ++j) idx[j] = j;
            std::stable_sort(idx.begin(), idx.end(), [&](unsigned a, unsigned b) { return route[a] < route[b]; });
            idx.resize(std::min(PK, Ki));
            keep[i] = idx;
        }
        std::vector<std::vector<std::pair<unsigned, unsigned>>> rev(n); // (rank, source)
        for (unsigned i = 0; i < n; ++i)
            for (unsigned r = 0; r < keep[i].size(); ++r) rev[nh[i].pool[keep[i][r]].id].push_back({r, i});
#pragma omp parallel for schedule(dynamic, 64)
        for (int w = 0; w < (int)n; ++w) std::sort(rev[w].begin(), rev[w].end());
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < (int)n; ++i) {
            auto &h = nh[i];
            h.nn_nsg.clear();
            size_t k = 0, j = 0;
            while (h.nn_nsg.size() < PK && (k < keep[i].size() || j < rev[i].size())) {
                if (k < keep[i].size()) h.nn_nsg.push_back(h.pool[keep[i][k++]]);
                if (j < rev[i].size()) {
                    const unsigned s = rev[i][j++].second;
                    h.nn_nsg.push_back(Nb(s, D(i, s), true));
                }
            }
        }
        update_nhoods();
    }

    // src/kgraph.cpp:3537-3584 (UpdateNhoods)
    void update_nhoods() {
#pragma omp parallel for schedule(dynamic, 100)
        for (int i = 0; i < (int)D.n; i++) {
            auto &h = nh[i];
            for (auto &e : h.nn_nsg)
                e.isnew = loopcount == 0 ? true
                                         : std::find(h.old_nsg.begin(), h.old_nsg.end(), e.id) == h.old_nsg.end();
            h.old_nsg.clear();
            for (auto &e : h.nn_nsg) h.old_nsg.push_back(e.id);
        }
    }

    // src/kgraph.cpp:2507-2561 (BridgeView_init)
    void bridge_init() {
        unsigned cur_loop = loopcount - 1;
        unsigned cur_L = std::min(P.search_L + cur_loop * P.step, MAXL);
#pragma omp parallel for
        for (int i = 0; i < (int)D.n; i++) {
            auto &h = nh[i];
            if (cur_loop == 0) {
                for (unsigned j = 0; j < h.L; j++) {
                    h.pool[j].flag = true;
                    h.pool[j].isnew = false;
                }
            } else {
                unsigned pre_L = std::min(P.search_L + (cur_loop - 1) * P.step, MAXL);
                for (unsigned j = 0; j < pre_L; j++) {
                    h.pool[j].flag = true;
                    h.pool[j].isnew = false;
                }
                for (unsigned j = pre_L; j < cur_L; j++) {
                    bool ex = h.pool[j].flag;
                    h.pool[j].isnew = ex;
                    h.pool[j].flag = true;
                }
                for (unsigned j = cur_L; j < h.L; j++) {
                    h.pool[j].flag = true;
                    h.pool[j].isnew = false;
                }
            }
            h.pool.resize(MAXL + 1);
            h.radius = h.pool.back().dist;
            h.rnn_new.clear();
            h.rnn_new_flag.clear();
        }
    }

    // src/kgraph.cpp:2562-2603 (BridgeView_update).  Pushes are collected per
    // source and appended in source order so one thread count gives one result.
    uint64_t bridge_update(bool capped) {
        unsigned nd = D.n, S_ = P.massq_S;
        unsigned Lp = std::min(P.search_L + (loopcount - 1) * P.step, MAXL);
        if (capped)
            for (auto &h : nh) {
                h.rnn_new.clear();
                h.rnn_new_flag.clear();
            }
        uint64_t count = 0;
        for (unsigned i = 0; i < nd; i++) {
            auto &h = nh[i];
            unsigned cnt = 0;
            for (unsigned j = 0; j < Lp && j < h.L && (cnt < S_ || !capped); j++) {
                if (h.pool[j].flag) {
                    unsigned id = h.pool[j].id;
                    nh[id].rnn_new.push_back(i);
                    nh[id].rnn_new_flag.push_back(h.pool[j].isnew);
                    h.pool[j].flag = false;
                    cnt++;
                }
            }
            count += cnt;
        }
        return count;
    }

    // src/kgraph.cpp:2604-2652 (BridgeView_join) with parallel_InsertIntoPool (:1539-1559)
    void bridge_join() {
        uint64_t cc = 0;
        unsigned nd = D.n;
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : cc)
        for (int i = 0; i < (int)nd; i++) {
            unsigned q = nd - i - 1;
            auto &h = nh[q];
            for (size_t k = 0; k < h.rnn_new.size(); k++) {
                unsigned id = h.rnn_new[k];
                bool ifnew = h.rnn_new_flag[k];
                for (auto &e : h.nn_nsg) {
                    unsigned w = e.id;
                    if (id == w) continue;
                    if (!ifnew && !e.isnew) continue;
                    cc++;
                    float dist = D(id, w);
                    auto &o = nh[id];
                    if (dist > o.radius) continue;
                    o.lock.lock();
                    Nb nn(w, dist, true);
                    nn.isnew = true;
                    unsigned l = (unsigned)insert_into_pool(o.pool.data(), o.L, nn);
                    if (l <= o.L) {
                        if (o.L + 1 < o.pool.size())
                            ++o.L;
                        else
                            o.radius = o.pool[o.L - 1].dist;
                    }
                    o.lock.unlock();
                }
            }
        }
        bridge_comps += cc;
    }

    // src/kgraph.cpp:2478-2506 (BridgeView)
    void bridge_view() {
        unsigned nd = D.n, S_ = P.massq_S;
        bridge_init();
        while (true) {
            uint64_t cnt = bridge_update(true);
            bool more = true;
            if ((float)cnt / nd / S_ < 0.5f) {
                cnt += bridge_update(false);
                more = false;
            }
            bridge_join();
            if (!more) break;
        }
        for (auto &h : nh) std::vector<unsigned>().swap(h.rnn_new);
    }

    // buildFastNSG / TauMNG / AlphaPG / HNSW layer: src/kgraph.cpp:3720-3966
    // Per-node pool search, src/kgraph.cpp:2340-2414 (poolSearch) driven by
    // inSearch (:3667-3688); the reference's builds call BridgeView in its
    // place (the inSearch calls at :3761, :3835, :3893, :3950 are commented
    // out).  Node q's pool is its beam: the entries at positions < cur_L are
    // expanded in pool order, each expansion inserting the unvisited graph
    // neighbours of the expanded node into the pool (InsertIntoPool), and the
    // scan restarts at the lowest position an insert landed at.  Only q's own
    // pool changes, so the result does not depend on thread timing.  Two
    // stated choices where the reference reads undefined state: the initial
    // radius is pool.back().dist (:2347), the overflow slot, which admits
    // exactly the inserts that reach pool[0, L) when it is taken as
    // pool[L - 1].dist for a full pool and +inf otherwise; positions at or
    // past the pool count are empty and not expanded.  Returns the distance
    // evaluations.
    uint64_t pool_search(unsigned q, std::vector<uint32_t> &mark, uint32_t stamp) {
        auto &h = nh[q];
        h.pool.resize(MAXL + 1);
        float radius = h.L >= MAXL ? h.pool[h.L - 1].dist : std::numeric_limits<float>::max();
        const unsigned cur_loop = loopcount - 1;
        const unsigned cur_L = std::min(P.search_L + cur_loop * P.step, MAXL);
        const unsigned pre_L = cur_loop == 0 ? 0 : std::min(P.search_L + (cur_loop - 1) * P.step, MAXL);
        for (unsigned t = 0; t < h.L; ++t) { // :2353-2384
            mark[h.pool[t].id] = stamp;
            h.pool[t].isnew = cur_loop > 0 && t >= pre_L && t < cur_L ? h.pool[t].flag : false;
            h.pool[t].flag = true;
        }
        uint64_t cc = 0;
        unsigned k = 0;
        while (k < cur_L) { // :2386-2410
            unsigned nk = cur_L;
            if (k < h.L && h.pool[k].flag) {
                h.pool[k].flag = false;
                const unsigned n = h.pool[k].id;
                for (const auto &e : nh[n].nn_nsg) {
                    const unsigned id = e.id;
                    if (mark[id] == stamp || id == q) continue;
                    mark[id] = stamp;
                    ++cc;
                    const float dist = D(q, id);
                    unsigned r = (unsigned)h.pool.size();
                    if (dist <= radius) { // parallel_InsertIntoPool, :1539-1559
                        Nb nn(id, dist, true);
                        nn.isnew = true;
                        r = (unsigned)insert_into_pool(&h.pool[0], h.L, nn);
                        if (r <= h.L) {
                            if (h.L + 1 < h.pool.size())
                                ++h.L;
                            else
                                radius = h.pool[h.L - 1].dist;
                        }
                    }
                    if (r < nk) nk = r;
                }
            }
            k = nk <= k ? nk : k + 1;
        }
        return cc;
    }

    // src/kgraph.cpp:3667-3688 (inSearch)
    uint64_t in_search() {
        uint64_t cc = 0;
#pragma omp parallel reduction(+ : cc)
        {
            std::vector<uint32_t> mark(D.n, 0);
            uint32_t stamp = 0;
#pragma omp for schedule(dynamic, 100)
            for (int i = 0; i < (int)D.n; ++i) cc += pool_search((unsigned)i, mark, ++stamp);
        }
        bridge_comps += cc;
        return cc;
    }

    void build() {
        nndescent();
        std::mt19937 rng(P.seed);
        std::srand(P.seed);
        st->loop_recall[0] = evaluate();
        st->nndescent_time = now() - t0;
        pruneAgain.assign(D.n, 1);
        init_nhoods();
        loopcount = 0;
        unsigned iters = P.loop_i + 1;
        for (unsigned iter = 1; iter <= iters; iter++) {
            double a = now();
            link();
            compute_ep(rng);
            double b = now();
            if (kind != KCNA_HNSW_LAYER) tree_grow(rng);
            double c = now();
            update_nhoods();
            if (loopcount < KCNA_MAX_LOOPS) {
                st->tree_grow_time[loopcount] = c - b;
                st->buildnsg_time[loopcount] = now() - a;
                st->con_time[loopcount] = now() - t0;
            }
            loopcount++;
            if (iter == iters) break;
            double s = now();
            if (P.refine == KCNA_REFINE_POOL_SEARCH)
                in_search();
            else
                bridge_view();
            if (loopcount - 1 < KCNA_MAX_LOOPS) st->search_time[loopcount - 1] = now() - s;
            if (loopcount <= KCNA_MAX_LOOPS) st->loop_recall[loopcount] = evaluate();
        }
        st->loops = loopcount;
        st->total_time = now() - t0;
        st->prune_comps = prune_comps;
        st->bridge_comps = bridge_comps;
        st->ep = ep;
        unsigned mx = 0, mn = ~0u;
        uint64_t sum = 0;
        width = 0;
        for (auto &h : nh) {
            unsigned s = (unsigned)h.nn_nsg.size();
            mx = std::max(mx, s);
            mn = std::min(mn, s);
            sum += s;
        }
        width = mx;
        st->width = mx;
        st->max_degree = mx;
        st->min_degree = mn;
        st->aod = (unsigned)(sum / std::max(1u, D.n)); // CalculateNSG, src/kgraph.cpp:2273-2293
    }
};

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

} // namespace kcnao

using namespace kcnao;

extern "C" {

void kcnao_params_default(kcna_params *p);

float kcnao_l2(const float *a, const float *b, uint32_t d) { return l2(a, b, d); }

// Exact k-NN of base rows ids[0..m) (self excluded), LinearSearch semantics.
int kcnao_knn(const float *X, uint64_t stride, uint32_t n, uint32_t d, const uint32_t *ids, uint32_t m, uint32_t k,
              uint32_t *out_ids, float *out_d, int nthreads) {
    if (k == 0 || k >= n) return KCNA_E_ARG;
    set_threads(nthreads);
    Data D{X, stride, n, d};
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < (int)m; ++i) {
        std::vector<Nb> nns;
        linear_search(D, ids[i], k, nns);
        for (uint32_t j = 0; j < k; ++j) {
            out_ids[(uint64_t)i * k + j] = nns[j].id;
            out_d[(uint64_t)i * k + j] = nns[j].dist;
        }
    }
    return 0;
}

// Exact k-NN of free query vectors (no self exclusion), SearchOracle::search semantics.
int kcnao_knn_queries(const float *X, uint64_t stride, uint32_t n, uint32_t d, const float *Q, uint64_t qstride,
                      uint32_t m, uint32_t k, uint32_t *out_ids, float *out_d, int nthreads) {
    if (k == 0 || k > n) return KCNA_E_ARG;
    set_threads(nthreads);
    Data D{X, stride, n, d};
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < (int)m; ++i) {
        std::vector<Nb> nns(k + 1);
        unsigned L = 0;
        const float *q = Q + (uint64_t)i * qstride;
        for (unsigned id = 0; id < n; ++id) {
            update_knn_list(&nns[0], L, Nb(id, D.q(q, id), true));
            if (L < k) ++L;
        }
        for (uint32_t j = 0; j < k; ++j) {
            out_ids[(uint64_t)i * k + j] = nns[j].id;
            out_d[(uint64_t)i * k + j] = nns[j].dist;
        }
    }
    return 0;
}

// Sequential try-insert of candidates into one pool (Nhood::parallel_try_insert).
// ids/dists/flags hold cap+1 slots; *L is the live count; *radius is updated.
int kcnao_pool_insert_seq(uint32_t *ids, float *dists, uint8_t *flags, uint32_t *L, uint32_t cap, float *radius,
                          const uint32_t *cid, const float *cd, uint32_t nc, uint32_t *ret) {
    Nhood h;
    h.pool.resize(cap + 1);
    for (uint32_t i = 0; i < *L; ++i) {
        h.pool[i].id = ids[i];
        h.pool[i].dist = dists[i];
        h.pool[i].flag = flags[i] != 0;
    }
    h.L = *L;
    h.radius = *radius;
    for (uint32_t c = 0; c < nc; ++c) {
        unsigned r = h.try_insert(cid[c], cd[c]);
        if (ret) ret[c] = r;
    }
    for (uint32_t i = 0; i < h.L; ++i) {
        ids[i] = h.pool[i].id;
        dists[i] = h.pool[i].dist;
        flags[i] = h.pool[i].flag;
    }
    *L = h.L;
    *radius = h.radius;
    return 0;
}

static void load_pools(Builder &B, const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap) {
    B.nh.clear();
    B.nh.resize(B.D.n);
    for (unsigned i = 0; i < B.D.n; ++i) {
        auto &h = B.nh[i];
        h.pool.resize(B.MAXL + 1);
        h.L = std::min(pcnt[i], B.MAXL);
        for (unsigned j = 0; j < h.L; ++j) {
            h.pool[j].id = pid[(uint64_t)i * cap + j];
            h.pool[j].dist = pd[(uint64_t)i * cap + j];
            h.pool[j].flag = false;
            h.pool[j].isnew = true;
        }
    }
}

static void store_graph(Builder &B, uint32_t *out_ids, float *out_d, uint32_t *out_deg, uint32_t width) {
    for (unsigned i = 0; i < B.D.n; ++i) {
        auto &g = B.nh[i].nn_nsg;
        uint32_t s = (uint32_t)std::min<size_t>(g.size(), width);
        out_deg[i] = (uint32_t)g.size();
        for (uint32_t j = 0; j < width; ++j) {
            out_ids[(uint64_t)i * width + j] = j < s ? g[j].id : 0xFFFFFFFFu;
            if (out_d) out_d[(uint64_t)i * width + j] = j < s ? g[j].dist : 0.f;
        }
    }
}

// Prune every pool (sync_prune of the given kind, or the CAGRA rank prune) into
// out (n x width).
int kcnao_prune(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
                const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap, uint32_t *out_ids,
                float *out_d, uint32_t *out_deg, uint32_t width, int nthreads) {
    set_threads(nthreads);
    kcna_stats st;
    memset(&st, 0, sizeof st);
    Builder B(Data{X, stride, n, d}, *p, kind, &st);
    B.MAXL = std::max(cap, std::max(std::max(p->L, p->K), std::max(p->search_L, p->search_K)));
    load_pools(B, pid, pd, pcnt, cap);
    if (kind == KCNA_CAGRA) {
        B.build_cagra();
    } else {
#pragma omp parallel for schedule(dynamic, 64)
        for (int q = 0; q < (int)n; ++q) B.sync_prune(q);
    }
    store_graph(B, out_ids, out_d, out_deg, width);
    return 0;
}

// Per-node pool search (inSearch of loop `loopcount`) of the given pools over
// the given graph; pools out (n x cap) and the distance evaluations.
int kcnao_pool_search(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
                      const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap,
                      const uint32_t *g_ids, const uint32_t *g_deg, uint32_t width, uint32_t loopcount,
                      uint32_t *out_ids, float *out_d, uint32_t *out_cnt, uint64_t *comps, int nthreads) {
    set_threads(nthreads);
    kcna_stats st;
    memset(&st, 0, sizeof st);
    Builder B(Data{X, stride, n, d}, *p, KCNA_NSG, &st);
    B.MAXL = cap;
    load_pools(B, pid, pd, pcnt, cap);
    for (unsigned i = 0; i < n; ++i) {
        B.nh[i].nn_nsg.clear();
        for (uint32_t j = 0; j < std::min(g_deg[i], width); ++j)
            B.nh[i].nn_nsg.push_back(Nb(g_ids[(uint64_t)i * width + j], 0.f, false));
    }
    B.loopcount = loopcount;
    *comps = B.in_search();
    for (unsigned i = 0; i < n; ++i) {
        const auto &h = B.nh[i];
        out_cnt[i] = h.L;
        for (uint32_t j = 0; j < cap; ++j) {
            out_ids[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].id : 0xFFFFFFFFu;
            out_d[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].dist : INFINITY;
        }
    }
    return 0;
}

// Full link (first loop: every node pruned from scratch) into out (n x width).
int kcnao_link(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
               const uint32_t *pid, const float *pd, const uint32_t *pcnt, uint32_t cap, uint32_t *out_ids,
               float *out_d, uint32_t *out_deg, uint32_t width, int nthreads) {
    set_threads(nthreads);
    kcna_stats st;
    memset(&st, 0, sizeof st);
    Builder B(Data{X, stride, n, d}, *p, kind, &st);
    B.MAXL = std::max(cap, std::max(std::max(p->L, p->K), std::max(p->search_L, p->search_K)));
    load_pools(B, pid, pd, pcnt, cap);
    B.pruneAgain.assign(n, 1);
    B.link();
    store_graph(B, out_ids, out_d, out_deg, width);
    return 0;
}

// Beam search (get_neighbors) of m queries over a caller graph from caller init ids.
int kcnao_beam_search(const float *X, uint64_t stride, uint32_t n, uint32_t d, const uint32_t *g_ids,
                      const uint32_t *g_deg, uint32_t width, const float *Q, uint64_t qstride, uint32_t m,
                      const uint32_t *init_ids, uint32_t L, uint32_t k, uint32_t *out_ids, float *out_d,
                      int nthreads) {
    set_threads(nthreads);
    kcna_params p;
    kcnao_params_default(&p);
    kcna_stats st;
    Builder B(Data{X, stride, n, d}, p, KCNA_NSG, &st);
    B.nh.resize(n);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned j = 0; j < std::min(g_deg[i], width); ++j) B.nh[i].nn_nsg.push_back(Nb(g_ids[(uint64_t)i * width + j], 0, true));
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < (int)m; ++i) {
        std::vector<unsigned> init(init_ids + (uint64_t)i * L, init_ids + (uint64_t)(i + 1) * L);
        std::vector<Nb> pool;
        B.beam_search(Q + (uint64_t)i * qstride, init, L, pool);
        for (uint32_t j = 0; j < k; ++j) {
            out_ids[(uint64_t)i * k + j] = j < L ? pool[j].id : 0xFFFFFFFFu;
            out_d[(uint64_t)i * k + j] = j < L ? pool[j].dist : 0.f;
        }
    }
    return 0;
}

// NN-descent only; pools out (n x cap) sorted, counts out.
int kcnao_nndescent(const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p, kcna_stats *st,
                    uint32_t *pool_ids, float *pool_d, uint32_t *pool_cnt, uint32_t cap, int nthreads) {
    set_threads(nthreads);
    memset(st, 0, sizeof *st);
    Builder B(Data{X, stride, n, d}, *p, KCNA_NSG, st);
    B.nndescent();
    st->loop_recall[0] = B.evaluate();
    st->nndescent_time = now() - B.t0;
    if (pool_ids)
        for (unsigned i = 0; i < n; ++i) {
            auto &h = B.nh[i];
            pool_cnt[i] = std::min(h.L, cap);
            for (unsigned j = 0; j < cap; ++j) {
                pool_ids[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].id : 0xFFFFFFFFu;
                pool_d[(uint64_t)i * cap + j] = j < h.L ? h.pool[j].dist : INFINITY;
            }
        }
    return 0;
}

// Full build of one kind; graph out (n x width, width >= max degree).
int kcnao_build(int kind, const float *X, uint64_t stride, uint32_t n, uint32_t d, const kcna_params *p,
                kcna_stats *st, uint32_t *g_ids, uint32_t *g_deg, uint32_t width, int use_prune2, int nthreads) {
    set_threads(nthreads);
    memset(st, 0, sizeof *st);
    Builder B(Data{X, stride, n, d}, *p, kind, st);
    B.use_prune2 = use_prune2 != 0;
    B.build();
    if (g_ids) store_graph(B, g_ids, nullptr, g_deg, width);
    return 0;
}

} // extern "C"

// Defaults of kgraph::IndexParams and the CLI (src/kgraph.h:12-40, src/fastnsg.cpp:53-94).
extern "C" void kcnao_params_default(kcna_params *p) {
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
