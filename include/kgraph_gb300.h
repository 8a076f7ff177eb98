/* kgraph_gb300.h - the FastKCNA C++ build interface (namespace kgraph) on the
 * GB300 library.
 *
 * Same names, parameter meaning and error types as the reference interface
 * (src/kgraph.h:12-304, exceptions :363-376), so code written against
 * kgraph::KGraph builds against this header after changing the include.  The
 * implementation (KGraph::create, fastkcna_gb300/host/kgraph_facade.cpp)
 * forwards every build to the C ABI of kcna.h; data must reach it through an
 * oracle that also implements kgraph::RowSource (kgraph::MatrixOracle in
 * kgraph_gb300_data.h does), any other oracle is rejected with
 * kgraph::invalid_argument because the device needs the rows, not a distance
 * callback.
 *
 * Parameter defaults are those of the reference (src/kgraph.h:12-37): they are
 * the CLI defaults callers rely on.
 */
#ifndef KGRAPH_GB300_H
#define KGRAPH_GB300_H

#include <stddef.h>

#include <stdexcept>
#include <string>
#include <vector>

namespace kgraph {

static unsigned const default_iterations = 30;
static unsigned const default_L = 100;
static unsigned const default_K = 25;
static unsigned const default_P = 100;
static unsigned const default_M = 0;
static unsigned const default_T = 1;
static unsigned const default_S = 10;
static unsigned const default_R = 100;
static unsigned const default_controls = 100;
static unsigned const default_seed = 2024;
static float const default_delta = 0.002f;
static float const default_recall = 0.95f;
static float const default_epsilon = 1e30f;
static unsigned const default_verbosity = 1;
static unsigned const default_nthreads = 40;
static unsigned const default_num0 = 100;
static unsigned const default_iter = 3;
static float const default_incr_r = 10.0f;
static unsigned const default_loop_i = 2;
static unsigned const default_nsgr = 50;
static unsigned const default_searchl = 40;
static unsigned const default_searchk = 500;
static unsigned const default_step = 10;
static unsigned const default_massqS = 10;
static float const default_tau = 0;
static float const default_angle = 60;
static unsigned const default_prune = 0;
enum { PRUNE_LEVEL_1 = 1, PRUNE_LEVEL_2 = 2 };
enum { REVERSE_AUTO = -1, REVERSE_NONE = 0 };
static int const default_reverse = REVERSE_NONE;

/* 0 silences progress output on stderr */
extern unsigned verbosity;

class invalid_argument : public std::invalid_argument {
public:
    using std::invalid_argument::invalid_argument;
};
class runtime_error : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};
class io_error : public runtime_error {
public:
    using runtime_error::runtime_error;
};

/* The data plugin (src/kgraph.h:63-81). */
class IndexOracle {
public:
    virtual ~IndexOracle() {}
    virtual unsigned size() const = 0;
    virtual unsigned dim() const = 0;
    virtual float operator()(unsigned i, unsigned j) const = 0;
    virtual float operator()(unsigned i, unsigned j, unsigned offset, unsigned dim) const = 0;
    virtual float operator()(const float *query, unsigned i) const = 0;
    virtual float computeDot(unsigned i, unsigned j) const = 0;
    virtual void computeSelfDotPtr() = 0;
    virtual float *Calcenter() const = 0;
    virtual unsigned data_size() const = 0;
    virtual void set_size(unsigned mysize) = 0;
};

/* Row access the device build needs: FP32 rows of data_size() x dim() with a
 * byte stride; size() may be a prefix of them (set_size). */
class RowSource {
public:
    virtual ~RowSource() {}
    virtual const float *rows() const = 0;
    virtual size_t row_stride_bytes() const = 0;
};

/* Query-side plugin (src/kgraph.h:87-106). */
class SearchOracle {
public:
    virtual ~SearchOracle() {}
    virtual unsigned size() const = 0;
    virtual float operator()(unsigned i) const = 0;
    /* brute force: the K nearest within epsilon, ascending; returns the count */
    unsigned search(unsigned K, float epsilon, unsigned *ids, float *dists = nullptr) const;
};

class KGraph {
public:
    struct IndexParams {
        unsigned nsg_R;
        unsigned search_L;
        unsigned search_K;
        unsigned step;
        float tau;
        float angle;
        unsigned nt;
        unsigned massq_S;
        unsigned loop_i;
        unsigned iterations;
        unsigned L;
        unsigned K;
        unsigned S;
        unsigned R;
        unsigned controls;
        unsigned seed;
        unsigned nthreads;
        float delta;
        float recall;
        unsigned prune;
        int reverse;
        unsigned num0;
        float incr_r;
        unsigned sl;
        unsigned iter;
        unsigned qid, Lcon, sidx, B, P;
        /* GB300 build options (no reference counterpart): screening precision
         * (0 FP32, 1 BF16), the learned initial graph (0 off, 1 on) and the
         * refinement between prune loops (0 BridgeView as the reference's
         * builds, 1 the per-node pool search, inSearch) */
        unsigned screen;
        unsigned learned_seed;
        unsigned refine;
        IndexParams()
            : nsg_R(default_nsgr), search_L(default_searchl), search_K(default_searchk), step(default_step),
              tau(default_tau), angle(default_angle), nt(0), massq_S(default_massqS), loop_i(default_loop_i),
              iterations(default_iterations), L(default_L), K(default_K), S(default_S), R(default_R),
              controls(default_controls), seed(default_seed), nthreads(default_nthreads), delta(default_delta),
              recall(default_recall), prune(default_prune), reverse(default_reverse), num0(default_num0),
              incr_r(default_incr_r), sl(0), iter(default_iter), qid(0), Lcon(0), sidx(0), B(0), P(default_P),
              screen(0), learned_seed(0), refine(0) {}
    };

    struct SearchParams {
        unsigned K, M, P, S, T;
        float epsilon;
        unsigned seed, init;
        SearchParams()
            : K(default_K), M(default_M), P(default_P), S(default_S), T(default_T), epsilon(default_epsilon),
              seed(1998), init(0) {}
    };

    enum { FORMAT_DEFAULT = 0, FORMAT_NO_DIST = 1 };

    struct IndexInfo {
        enum StopCondition { ITERATION = 0, DELTA, RECALL } stop_condition;
        unsigned iterations;
        float cost;
        float recall;
        float accuracy;
        float delta;
        float M;
    };

    struct SearchInfo {
        float cost;
        unsigned updates;
    };

    virtual ~KGraph() {}
    /* NSG file of the current graph (u32 width, u32 ep, per node u32 degree + ids) */
    virtual void load(char const *path) = 0;
    virtual void save(char const *path, int format = FORMAT_DEFAULT) const = 0;
    /* Builds (src/kgraph.h:230-234).  nsg_name: index file written when
     * non-empty; res_name: CSV of timings appended to when non-empty. */
    virtual void buildFastNSG(IndexOracle const &oracle, IndexParams const &param, IndexInfo *info = 0,
                              const char *nsg_name = 0, const char *res_name = 0) = 0;
    virtual void buildFastTauMNG(IndexOracle const &oracle, IndexParams const &param, IndexInfo *info = 0,
                                 const char *nsg_name = 0, const char *res_name = 0) = 0;
    virtual void buildFastAlphaPG(IndexOracle const &oracle, IndexParams const &param, IndexInfo *info = 0,
                                  const char *nsg_name = 0, const char *res_name = 0) = 0;
    /* One HNSW layer over the first oracle.size() rows.  level > 0: writes the
     * layer's lists into linkLists_[i] + (level-1) * (4 + 4*nsg_R); level 0:
     * keeps the graph for FatherSwapHNSWLayer0.  *ep_ptr = the layer's entry. */
    virtual void buildFastHNSW(IndexOracle const &oracle, IndexParams const &param, IndexInfo *info,
                               const char *nsg_name, const char *res_name, char *&data_level0_memory_,
                               char **linkLists_ = 0, unsigned level = 0, unsigned *ep_ptr = 0,
                               size_t size_data_per_element_ = 0) = 0;
    /* Level-0 lists into hnswlib's level-0 block (element size 4 + 4*nsg_R + 4*dim + 8). */
    virtual void FatherSwapHNSWLayer0(IndexOracle const &oracle, IndexParams const &params,
                                      char *&data_level0_memory_) = 0;
    /* KGraph's own index pruning levels: not part of the FastKCNA build path;
     * throws kgraph::runtime_error. */
    virtual void prune(IndexOracle const &oracle, unsigned level) = 0;
    unsigned search(SearchOracle const &oracle, SearchParams const &params, unsigned *ids,
                    SearchInfo *info = 0) const {
        return search(oracle, params, ids, nullptr, info);
    }
    /* Greedy search of the built graph through a SearchOracle (host). */
    virtual unsigned search(SearchOracle const &oracle, SearchParams const &params, unsigned *ids, float *dists,
                            SearchInfo *info) const = 0;
    static KGraph *create();
    static char const *version();
    /* The pool (candidate list) of node id after the last build. */
    virtual void get_nn(unsigned id, unsigned *nns, unsigned *M, unsigned *L) const { get_nn(id, nns, nullptr, M, L); }
    virtual void get_nn(unsigned id, unsigned *nns, float *dists, unsigned *M, unsigned *L) const = 0;
    virtual void reverse(int) = 0;
    virtual void swapResult(std::vector<std::vector<int> > &knng) = 0;
    virtual void swapResult(std::vector<std::vector<unsigned> > &knng) = 0;
};

} // namespace kgraph

#endif
