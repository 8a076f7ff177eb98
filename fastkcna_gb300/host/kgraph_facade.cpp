// kgraph_facade.cpp - kgraph::KGraph (include/kgraph_gb300.h) on the kcna C ABI.
//
// KGraph::create() returns a KGraphCuda: every build uploads the oracle's rows
// (once; an HNSW layer over a prefix of the same rows only moves the prefix
// with kcna_set_size), runs kcna_build on the device, copies the resulting
// graph to the host and writes the files the reference writes: the NSG index
// (src/kgraph.cpp:1704-1724) and the CSV of timings (SaveResult,
// src/kgraph.cpp:1725-1806, same rows).  Status codes become the reference's
// exception types: KCNA_E_ARG -> kgraph::invalid_argument, KCNA_E_IO ->
// kgraph::io_error, anything else -> kgraph::runtime_error.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "kcna.h"
#include "kgraph_gb300.h"
#include "kgraph_gb300_data.h"

namespace kgraph {

unsigned verbosity = default_verbosity;

unsigned SearchOracle::search(unsigned K, float epsilon, unsigned *ids, float *dists) const {
    std::vector<std::pair<float, unsigned> > all;
    all.reserve(size());
    for (unsigned i = 0; i < size(); ++i) {
        const float d = (*this)(i);
        if (d <= epsilon) all.emplace_back(d, i);
    }
    const unsigned k = std::min<unsigned>(K, (unsigned)all.size());
    std::partial_sort(all.begin(), all.begin() + k, all.end());
    for (unsigned i = 0; i < k; ++i) {
        ids[i] = all[i].second;
        if (dists) dists[i] = all[i].first;
    }
    return k;
}

namespace {

[[noreturn]] void raise(kcna_ctx *c, kcna_status s, const char *what) {
    std::string msg = std::string(what) + ": " + (c ? kcna_last_error(c) : "no context");
    if (s == KCNA_E_ARG) throw invalid_argument(msg);
    if (s == KCNA_E_IO) throw io_error(msg);
    throw runtime_error(msg);
}

kcna_params to_params(const KGraph::IndexParams &p) {
    kcna_params k;
    kcna_params_default(&k);
    k.K = p.K;
    k.L = p.L;
    k.S = p.S;
    k.R = p.R;
    k.iterations = p.iterations;
    k.controls = p.controls;
    k.seed = p.seed;
    k.nthreads = p.nthreads;
    k.delta = p.delta;
    k.recall = p.recall;
    k.nsg_R = p.nsg_R;
    k.search_L = p.search_L;
    k.search_K = p.search_K;
    k.step = p.step;
    k.massq_S = p.massq_S;
    k.loop_i = p.loop_i;
    k.tau = p.tau;
    k.angle = p.angle;
    k.screen = p.screen;
    k.learned_seed = p.learned_seed;
    k.refine = p.refine;
    k.verbosity = verbosity;
    return k;
}

// SaveResult rows (src/kgraph.cpp:1738-1804); PG_type 0 NSG, 1 tau-MNG, 2 HNSW layer, 3 alpha-PG
void write_result(const char *path, int pg_type, const KGraph::IndexParams &p, const kcna_stats &st) {
    std::ofstream o(path, std::ios::out | std::ios::app);
    if (!o) return;
    o << "PG_type,K,L,S,R,I,searchL,searchK,nsgR,massqS,tau,angle,step\n";
    o << pg_type << "," << p.K << "," << p.L << "," << p.S << "," << p.R << "," << p.iterations << "," << p.search_L
      << "," << p.search_K << "," << p.nsg_R << "," << p.massq_S << "," << p.tau << "," << p.angle << "," << p.step
      << ",\n";
    auto row = [&o](const char *name, const double *v, unsigned n) {
        o << name << ",";
        for (unsigned i = 0; i < n; ++i) o << v[i] << ",";
        o << "\n";
    };
    const unsigned loops = std::min<unsigned>(st.loops, KCNA_MAX_LOOPS);
    std::vector<double> kt(1, st.nndescent_time), rec;
    for (unsigned i = 0; i + 1 < loops; ++i) kt.push_back(st.con_time[i] + st.search_time[i]);
    for (unsigned i = 0; i < loops; ++i) rec.push_back(st.loop_recall[i]);
    row("kgraph time", kt.data(), (unsigned)kt.size());
    row("recall", rec.data(), (unsigned)rec.size());
    row("prune time", st.prune_time, loops);
    row("inter time", st.inter_time, loops);
    row("tree_grow time", st.tree_grow_time, pg_type == 2 ? 0 : loops);
    row("buildnsg time", st.buildnsg_time, loops);
    row("search time", st.search_time, loops ? loops - 1 : 0);
    row("con time", st.con_time, loops);
    std::vector<double> pcc(loops, (double)st.prune_comps), scc(loops ? loops - 1 : 0, (double)st.bridge_comps);
    row("prune cc", pcc.data(), (unsigned)pcc.size());
    row("search cc", scc.data(), (unsigned)scc.size());
    o << "AOD," << st.aod << "\n";
    o << "final_prune_time,0\n";
}

class KGraphCuda : public KGraph {
    kcna_ctx *ctx_ = nullptr;
    const float *rows_ = nullptr; // rows currently on the device
    unsigned rows_n_ = 0, rows_d_ = 0;
    size_t rows_stride_ = 0;
    std::vector<std::vector<unsigned> > graph_; // last graph (host)
    unsigned ep_ = 0, width_ = 0;
    std::vector<std::vector<unsigned> > temp_graph_; // level-0 lists kept for FatherSwapHNSWLayer0
    // pools copied to the host on the first get_nn after a build
    mutable std::vector<uint32_t> pool_ids_, pool_cnt_;
    mutable std::vector<float> pool_d_;
    mutable uint32_t pool_cap_ = 0;
    bool pools_on_device_ = false;

    void ensure_ctx() {
        if (ctx_) return;
        const char *dev = getenv("KCNA_DEVICE");
        kcna_status s = kcna_create(&ctx_, dev ? atoi(dev) : 0);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_create");
    }
    void put_rows(IndexOracle const &oracle) {
        const RowSource *rs = dynamic_cast<const RowSource *>(&oracle);
        if (!rs) throw invalid_argument("oracle must implement kgraph::RowSource (use kgraph::MatrixOracle)");
        ensure_ctx();
        if (rs->rows() != rows_ || oracle.data_size() != rows_n_ || oracle.dim() != rows_d_ ||
            rs->row_stride_bytes() != rows_stride_) {
            kcna_status s = kcna_upload(ctx_, rs->rows(), oracle.data_size(), oracle.dim(), rs->row_stride_bytes());
            if (s != KCNA_OK) raise(ctx_, s, "kcna_upload");
            rows_ = rs->rows();
            rows_n_ = oracle.data_size();
            rows_d_ = oracle.dim();
            rows_stride_ = rs->row_stride_bytes();
        }
        kcna_status s = kcna_set_size(ctx_, oracle.size());
        if (s != KCNA_OK) raise(ctx_, s, "kcna_set_size");
    }
    void fetch_graph(unsigned n) {
        uint32_t ep = 0, w = 0;
        kcna_status s = kcna_get_graph(ctx_, nullptr, nullptr, &ep, &w);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_get_graph");
        std::vector<uint32_t> ids((size_t)n * w), deg(n);
        s = kcna_get_graph(ctx_, ids.data(), deg.data(), &ep, &w);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_get_graph");
        graph_.assign(n, {});
        width_ = 0;
        for (unsigned i = 0; i < n; ++i) {
            graph_[i].assign(ids.begin() + (size_t)i * w, ids.begin() + (size_t)i * w + deg[i]);
            width_ = std::max<unsigned>(width_, deg[i]);
        }
        ep_ = ep;
        pool_cap_ = 0; // pools stay on the device until get_nn asks for them
        pools_on_device_ = true;
    }
    void fetch_pools() const {
        if (!pools_on_device_ || !ctx_) throw invalid_argument("get_nn: no pools (build first)");
        uint32_t cap = 0;
        kcna_status s = kcna_pool_capacity(ctx_, &cap);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_pool_capacity");
        const size_t n = graph_.size();
        pool_ids_.resize(n * cap);
        pool_d_.resize(n * cap);
        pool_cnt_.resize(n);
        s = kcna_get_pools(ctx_, pool_ids_.data(), pool_d_.data(), pool_cnt_.data(), cap);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_get_pools");
        pool_cap_ = cap;
    }
    kcna_stats run(kcna_kind kind, IndexOracle const &oracle, IndexParams const &param, IndexInfo *info,
                   const char *nsg_name, const char *res_name, int pg_type) {
        kcna_stats st;
        memset(&st, 0, sizeof st);
        if (oracle.size() < 3) { // one or two nodes (a top HNSW layer): nothing to search, link both ways
            if (!dynamic_cast<const RowSource *>(&oracle)) throw invalid_argument("oracle must implement kgraph::RowSource");
            graph_.assign(oracle.size(), {});
            if (oracle.size() == 2) graph_ = {{1u}, {0u}};
            ep_ = 0;
            width_ = oracle.size() - 1;
            pool_cap_ = 0;
            pools_on_device_ = false;
            if (info) memset(info, 0, sizeof *info);
            if (nsg_name && *nsg_name) save(nsg_name, 0);
            return st;
        }
        put_rows(oracle);
        kcna_params kp = to_params(param);
        kcna_status s = kcna_build(ctx_, &kp, kind, &st);
        if (s != KCNA_OK) raise(ctx_, s, "kcna_build");
        fetch_graph(oracle.size());
        if (info) {
            info->stop_condition = (IndexInfo::StopCondition)st.stop_condition;
            info->iterations = st.iterations;
            const double n = oracle.size();
            info->cost = n > 1 ? (float)(st.n_comps / (n * (n - 1) / 2)) : 0.f;
            info->recall = st.loop_recall[std::min<unsigned>(st.loops, KCNA_MAX_LOOPS)];
            info->accuracy = 0.f;
            info->delta = st.iterations ? st.iter_delta[st.iterations - 1] : 0.f;
            info->M = 0.f;
        }
        if (nsg_name && *nsg_name) {
            s = kcna_write_nsg(ctx_, nsg_name);
            if (s != KCNA_OK) raise(ctx_, s, "kcna_write_nsg");
        }
        if (res_name && *res_name) write_result(res_name, pg_type, param, st);
        if (verbosity)
            fprintf(stderr, "kcna: %s build of %u rows: %.3f s, control recall %.4f, AOD %u\n", kcna_version(),
                    oracle.size(), st.total_time, (double)st.loop_recall[std::min<unsigned>(st.loops, KCNA_MAX_LOOPS)],
                    st.aod);
        return st;
    }

public:
    ~KGraphCuda() override {
        if (ctx_) kcna_destroy(ctx_);
    }
    void buildFastNSG(IndexOracle const &o, IndexParams const &p, IndexInfo *info, const char *nsg_name,
                      const char *res_name) override {
        run(KCNA_NSG, o, p, info, nsg_name, res_name, 0);
    }
    void buildFastTauMNG(IndexOracle const &o, IndexParams const &p, IndexInfo *info, const char *nsg_name,
                         const char *res_name) override {
        run(KCNA_TAUMNG, o, p, info, nsg_name, res_name, 1);
    }
    void buildFastAlphaPG(IndexOracle const &o, IndexParams const &p, IndexInfo *info, const char *nsg_name,
                          const char *res_name) override {
        run(KCNA_ALPHAPG, o, p, info, nsg_name, res_name, 3);
    }
    void buildFastHNSW(IndexOracle const &o, IndexParams const &p, IndexInfo *info, const char *,
                       const char *res_name, char *&, char **linkLists_, unsigned level, unsigned *ep_ptr,
                       size_t) override {
        run(KCNA_HNSW_LAYER, o, p, info, nullptr, res_name, 2);
        if (ep_ptr) *ep_ptr = ep_;
        if (level > 0) { // SwapHNSWLayer (src/kgraph.cpp:3598-3614)
            if (!linkLists_) throw invalid_argument("buildFastHNSW: level > 0 needs linkLists_");
            const size_t per = (size_t)p.nsg_R * 4 + 4;
            for (unsigned i = 0; i < o.size(); ++i) {
                const std::vector<unsigned> &g = graph_[i];
                if (g.size() > p.nsg_R) throw runtime_error("buildFastHNSW: layer degree above nsg_R");
                char *cll = linkLists_[i] + (size_t)(level - 1) * per;
                const uint16_t cnt = (uint16_t)g.size();
                memcpy(cll, &cnt, 2);
                if (!g.empty()) memcpy(cll + 4, g.data(), g.size() * 4);
            }
        } else {
            temp_graph_ = graph_;
        }
    }
    // level-0 lists into hnswlib's level-0 block (src/kgraph.cpp:499-520)
    void FatherSwapHNSWLayer0(IndexOracle const &o, IndexParams const &p, char *&data_level0_memory_) override {
        const size_t links0 = (size_t)p.nsg_R * 4 + 4;
        const size_t per = links0 + 4 * (size_t)o.dim() + 8;
        if (temp_graph_.size() < o.size()) throw runtime_error("FatherSwapHNSWLayer0: no level-0 graph");
        for (unsigned i = 0; i < o.size(); ++i) {
            const std::vector<unsigned> &g = temp_graph_[i];
            if (g.size() > p.nsg_R) throw runtime_error("FatherSwapHNSWLayer0: degree above maxM0");
            char *cll = data_level0_memory_ + (size_t)i * per;
            const uint16_t cnt = (uint16_t)g.size();
            memcpy(cll, &cnt, 2);
            if (!g.empty()) memcpy(cll + 4, g.data(), g.size() * 4);
        }
    }
    void load(char const *path) override {
        std::ifstream is(path, std::ios::binary);
        if (!is) throw io_error(path);
        uint32_t w = 0, ep = 0;
        is.read((char *)&w, 4);
        is.read((char *)&ep, 4);
        graph_.clear();
        uint32_t k = 0;
        while (is.read((char *)&k, 4)) {
            std::vector<unsigned> row(k);
            if (k && !is.read((char *)row.data(), (std::streamsize)k * 4)) throw io_error(path);
            graph_.push_back(std::move(row));
        }
        width_ = w;
        ep_ = ep;
    }
    void save(char const *path, int) const override { // SaveNsg layout (src/kgraph.cpp:1704-1724)
        std::ofstream os(path, std::ios::binary);
        if (!os) throw io_error(path);
        const uint32_t w = width_, ep = ep_;
        os.write((const char *)&w, 4);
        os.write((const char *)&ep, 4);
        for (const std::vector<unsigned> &g : graph_) {
            const uint32_t k = (uint32_t)g.size();
            os.write((const char *)&k, 4);
            if (k) os.write((const char *)g.data(), (std::streamsize)k * 4);
        }
        if (!os) throw io_error(path);
    }
    void prune(IndexOracle const &, unsigned) override {
        throw runtime_error("KGraph::prune levels are not part of the FastKCNA build path");
    }
    // greedy beam search of the host graph from the entry point, pool of
    // max(K, P) entries, distances from the oracle (host, one query)
    unsigned search(SearchOracle const &oracle, SearchParams const &params, unsigned *ids, float *dists,
                    SearchInfo *info) const override {
        if (graph_.empty()) throw runtime_error("search: no graph");
        const unsigned L = std::max(params.K, params.P);
        std::vector<std::pair<float, unsigned> > pool; // sorted ascending
        std::vector<char> seen(graph_.size(), 0), done(graph_.size(), 0);
        unsigned evals = 0;
        auto consider = [&](unsigned id) {
            if (id >= graph_.size() || seen[id]) return;
            seen[id] = 1;
            const float d = oracle(id);
            ++evals;
            if (pool.size() >= L && d >= pool.back().first) return;
            pool.insert(std::upper_bound(pool.begin(), pool.end(), std::make_pair(d, id)), std::make_pair(d, id));
            if (pool.size() > L) pool.pop_back();
        };
        consider(ep_);
        for (unsigned nb : graph_[ep_]) consider(nb);
        for (size_t i = 0; i < pool.size();) {
            const unsigned u = pool[i].second;
            if (done[u]) {
                ++i;
                continue;
            }
            done[u] = 1;
            for (unsigned nb : graph_[u]) consider(nb);
            i = 0; // continue from the best unexpanded entry
        }
        const unsigned k = std::min<unsigned>(params.K, (unsigned)pool.size());
        for (unsigned i = 0; i < k; ++i) {
            ids[i] = pool[i].second;
            if (dists) dists[i] = pool[i].first;
        }
        if (info) {
            info->cost = graph_.empty() ? 0.f : (float)evals / graph_.size();
            info->updates = 0;
        }
        return k;
    }
    void get_nn(unsigned id, unsigned *nns, float *dists, unsigned *M, unsigned *L) const override {
        if (!pool_cap_) fetch_pools();
        if (id >= pool_cnt_.size()) throw invalid_argument("get_nn: id out of range");
        const uint32_t c = pool_cnt_[id];
        for (uint32_t j = 0; j < c; ++j) {
            nns[j] = pool_ids_[(size_t)id * pool_cap_ + j];
            if (dists) dists[j] = pool_d_[(size_t)id * pool_cap_ + j];
        }
        if (M) *M = c;
        if (L) *L = c;
    }
    void reverse(int) override { throw runtime_error("KGraph::reverse is not part of the FastKCNA build path"); }
    void swapResult(std::vector<std::vector<int> > &knng) override {
        knng.assign(graph_.size(), {});
        for (size_t i = 0; i < graph_.size(); ++i) knng[i].assign(graph_[i].begin(), graph_[i].end());
    }
    void swapResult(std::vector<std::vector<unsigned> > &knng) override { knng = graph_; }
};

} // namespace

KGraph *KGraph::create() { return new KGraphCuda(); }
char const *KGraph::version() { return kcna_version(); }

} // namespace kgraph

// Level assignment used by fasthnsw (kgraph::hnsw_levels), exported so that it
// can be checked against the reference's Matrix::getlevel without a GPU.
extern "C" int kgraph_gb300_levels(uint32_t n, uint32_t M, uint32_t seed, int *data2file, int *points_num,
                                   uint32_t max_levels, uint32_t *nlevels) {
    std::vector<int> level, d2f, pn;
    kgraph::hnsw_levels(n, M, seed, level, d2f, pn);
    if (pn.size() > max_levels) return 1;
    std::copy(d2f.begin(), d2f.end(), data2file);
    std::copy(pn.begin(), pn.end(), points_num);
    *nlevels = (uint32_t)pn.size();
    return 0;
}
