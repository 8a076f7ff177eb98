// fastkcna_cli.cpp - the fastnsg / fasttaumng / fastalphapg / fasthnsw /
// fastnsw command lines on the GB300 library.
//
// One source, built once per tool with -DKCNA_CLI=<1..5>.  Same flags,
// defaults, positional arguments and outputs as the reference tools
// (src/fastnsg.cpp:53-94 and its siblings): the index file (NSG layout, or
// hnswlib layout for fasthnsw/fastnsw, src/fasthnsw.cpp:317-342) and the CSV
// of timings.  Arguments are parsed here without Boost: "--name value",
// "--name=value", "-K value" and "-K100" are accepted.
//
// GB300 additions: --screen fp32|bf16 (row precision / Gram-tile join),
// --learned 0|1 (learned initial graph), --refine bridge|pool (the
// refinement between prune loops), --device N, and --print-params,
// which prints the parsed parameters as JSON and exits without touching a GPU.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/resource.h>

#include <chrono>
#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "kgraph_gb300.h"
#include "kgraph_gb300_data.h"

#ifndef KCNA_CLI
#define KCNA_CLI 1
#endif
// 1 fastnsg, 2 fasttaumng, 3 fastalphapg, 4 fasthnsw, 5 fastnsw
static const char *const kToolNames[] = {"", "fastnsg", "fasttaumng", "fastalphapg", "fasthnsw", "fastnsw"};

using namespace kgraph;

namespace {

struct Opt {
    const char *name;  // long name
    const char *alias; // second long name or single-letter short name, may be ""
    bool flag;         // takes no value
    const char *help;
};

const Opt kVisible[] = {
    {"help", "h", true, "produce help message."},
    {"version", "v", true, "print version information."},
    {"data", "", false, "data name"},
    {"output", "", false, "output path"},
    {"result", "", false, "result path"},
    {"K", "K", false, "number of nearest neighbor"},
    {"nthreads", "nt", false, "number of threads"},
    {"controls", "C", false, "number of control points"},
    {"nsg_R", "", false, ""},
    {"loop_i", "", false, ""},
    {"search_L", "", false, ""},
    {"search_K", "", false, ""},
    {"massq_S", "", false, ""},
    {"angle", "", false, ""},
    {"step", "", false, ""},
    {"tau", "", false, ""},
};
const Opt kHidden[] = {
    {"iterations", "I", false, ""},
    {"S", "S", false, ""},
    {"R", "R", false, ""},
    {"L", "L", false, ""},
    {"delta", "", false, ""},
    {"recall", "", false, ""},
    {"prune", "", false, ""},
    {"reverse", "", false, ""},
    {"noise", "", false, "noise"},
    {"seed", "", false, ""},
    {"dim", "D", false, "dimension, see format"},
    {"skip", "", false, "see format"},
    {"gap", "", false, "see format"},
    {"raw", "", true, "read raw binary file, need to specify D."},
    {"synthetic", "", false, "generate synthetic data, specify number of points"},
    {"l2norm", "", true, "l2-normalize data, so as to mimic cosine similarity"},
    {"screen", "", false, "GB300: row precision fp32 | bf16"},
    {"learned", "", false, "GB300: 1 = learned initial graph"},
    {"refine", "", false, "GB300: refinement between prune loops, bridge | pool"},
    {"device", "", false, "GB300: CUDA device"},
    {"print-params", "", true, "GB300: print the parsed parameters as JSON and exit"},
};

const Opt *find_opt(const std::string &n) {
    for (const Opt &o : kVisible)
        if (n == o.name || (*o.alias && n == o.alias)) return &o;
    for (const Opt &o : kHidden)
        if (n == o.name || (*o.alias && n == o.alias)) return &o;
    return nullptr;
}

void usage(const char *tool) {
    printf("Usage: %s [OTHER OPTIONS]... INPUT [OUTPUT]\nGeneral options:\n", tool);
    for (const Opt &o : kVisible) printf("  --%-12s %s\n", o.name, o.help);
    printf("Expert options:\n");
    for (const Opt &o : kHidden) printf("  --%-12s %s\n", o.name, o.help);
}

// name -> value ("" for flags); positionals in order
struct Args {
    std::map<std::string, std::string> v;
    std::vector<std::string> pos;
    bool has(const char *n) const { return v.count(n) != 0; }
};

Args parse(int argc, char **argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        std::string s = argv[i];
        if (s.size() < 2 || s[0] != '-') {
            a.pos.push_back(s);
            continue;
        }
        std::string name, val;
        bool inline_val = false;
        if (s[1] == '-') { // --name or --name=value
            name = s.substr(2);
            size_t eq = name.find('=');
            if (eq != std::string::npos) {
                val = name.substr(eq + 1);
                name = name.substr(0, eq);
                inline_val = true;
            }
        } else { // -K 100, -K100, -nt 8
            name = s.substr(1);
            if (!find_opt(name) && name.size() > 1 && find_opt(name.substr(0, 1))) {
                val = name.substr(1);
                name = name.substr(0, 1);
                inline_val = true;
            }
        }
        const Opt *o = find_opt(name);
        if (!o) throw invalid_argument("unrecognised option '" + s + "'");
        if (!o->flag && !inline_val) {
            if (i + 1 >= argc) throw invalid_argument("option '" + s + "' needs a value");
            val = argv[++i];
        }
        a.v[o->name] = val;
    }
    if (!a.has("data") && a.pos.size() > 0) a.v["data"] = a.pos[0];
    if (!a.has("output") && a.pos.size() > 1) a.v["output"] = a.pos[1];
    return a;
}

template <typename T>
void get(const Args &a, const char *n, T &dst) {
    auto it = a.v.find(n);
    if (it == a.v.end()) return;
    char *end = nullptr;
    const double x = strtod(it->second.c_str(), &end);
    if (end == it->second.c_str() || *end) throw invalid_argument(std::string("bad value for --") + n);
    dst = (T)x;
}

long peak_memory_mb() {
    struct rusage r;
    getrusage(RUSAGE_SELF, &r);
    return r.ru_maxrss / 1024;
}

void print_params(const KGraph::IndexParams &p, const std::string &data, const std::string &out,
                  const std::string &res) {
    printf("{\"tool\": \"%s\", \"data\": \"%s\", \"output\": \"%s\", \"result\": \"%s\", \"K\": %u, \"L\": %u, "
           "\"S\": %u, \"R\": %u, \"iterations\": %u, \"controls\": %u, \"seed\": %u, \"nthreads\": %u, "
           "\"delta\": %g, \"recall\": %g, \"nsg_R\": %u, \"search_L\": %u, \"search_K\": %u, \"step\": %u, "
           "\"massq_S\": %u, \"loop_i\": %u, \"tau\": %g, \"angle\": %g, \"prune\": %u, \"reverse\": %d, "
           "\"screen\": %u, \"learned_seed\": %u, \"refine\": %u}\n",
           kToolNames[KCNA_CLI], data.c_str(), out.c_str(), res.c_str(), p.K, p.L, p.S, p.R, p.iterations,
           p.controls, p.seed, p.nthreads, (double)p.delta, (double)p.recall, p.nsg_R, p.search_L, p.search_K,
           p.step, p.massq_S, p.loop_i, (double)p.tau, (double)p.angle, p.prune, p.reverse, p.screen,
           p.learned_seed, p.refine);
}

template <typename T>
void write_pod(std::ostream &o, const T &v) {
    o.write((const char *)&v, sizeof(T));
}

// fasthnsw / fastnsw: layers from the top level down on prefixes of the
// level-ordered rows, then hnswlib's file (src/fasthnsw.cpp:204-342).
int run_hnsw(KGraph::IndexParams params, Matrix<float> &data, std::vector<int> &labels, std::vector<int> &points_num,
             double level_secs, const std::string &output_path, const std::string &res_path) {
    const auto t0 = std::chrono::high_resolution_clock::now();
    {
        std::ofstream r(res_path, std::ios::out | std::ios::app);
        if (r) r << "start*****\nget_level_time," << level_secs << "\n";
    }
    std::vector<int> levels;
    for (int l = (int)points_num.size() - 1; l >= 0; --l)
        for (int j = 0; j < points_num[l]; ++j) levels.push_back(l);
    const size_t n = data.size(), dim = data.dim();
    const size_t M = params.nsg_R, maxM = params.nsg_R, maxM0 = 2 * (size_t)params.nsg_R;
    const size_t links = maxM * 4 + 4, links0 = maxM0 * 4 + 4;
    const size_t per_elem = links0 + 4 * dim + 8, offset_data = links0, label_offset = links0 + 4 * dim;
    const size_t offset_level0 = 0, ef_construction = params.search_K;
    const int maxlevel = levels.empty() ? 0 : levels[0];
    const double mult = 1 / std::log(1.0 * M);
    std::vector<char *> link_lists(n, nullptr);
    for (size_t i = 0; i < n && levels[i] > 0; ++i) link_lists[i] = (char *)calloc(links * levels[i] + 1, 1);
    MatrixOracle<Matrix<float>, metric::l2sqr> oracle(data);
    KGraph *kg = KGraph::create();
    KGraph::IndexInfo info;
    unsigned ep = 0, layer_ep = 0;
    char *level0 = nullptr;
    unsigned size = 0;
    for (int level = (int)points_num.size() - 1; level >= 0; --level) {
        size += points_num[level];
        oracle.set_size(size);
        if (size == 1 && level > 0) { // a lone top node: empty list on this level
            memset(link_lists[0] + (size_t)(level - 1) * links, 0, 2);
            if (level == (int)points_num.size() - 1) ep = 0;
            continue;
        }
        if (level > 0) {
            kg->buildFastHNSW(oracle, params, &info, output_path.c_str(), res_path.c_str(), level0, link_lists.data(),
                              (unsigned)level, &layer_ep);
        } else {
            params.nsg_R *= 2;
            kg->buildFastHNSW(oracle, params, &info, output_path.c_str(), res_path.c_str(), level0, link_lists.data(),
                              0, &layer_ep, per_elem);
            level0 = (char *)calloc(n * per_elem, 1);
            kg->FatherSwapHNSWLayer0(oracle, params, level0);
        }
        if (level == (int)points_num.size() - 1) ep = layer_ep;
    }
    delete kg;
    for (size_t i = 0; i < n; ++i) {
        const size_t label = (size_t)labels[i];
        memcpy(level0 + i * per_elem + offset_data, data[(unsigned)i], 4 * dim);
        memcpy(level0 + i * per_elem + label_offset, &label, sizeof label);
    }
    const double secs = std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - t0).count() + level_secs;
    printf("%s indexing time: %f\n", kToolNames[KCNA_CLI], secs);
    {
        std::ofstream r(res_path, std::ios::out | std::ios::app);
        if (r) r << kToolNames[KCNA_CLI] << " indexing time," << secs << "\nend*****\n\n";
    }
    std::ofstream out(output_path, std::ios::binary);
    if (!out) throw io_error(output_path);
    write_pod(out, offset_level0);
    write_pod(out, n);              // max_elements
    write_pod(out, n);              // cur_element_count
    write_pod(out, per_elem);       // size_data_per_element
    write_pod(out, label_offset);
    write_pod(out, offset_data);
    write_pod(out, maxlevel);
    write_pod(out, ep);
    write_pod(out, maxM);
    write_pod(out, maxM0);
    write_pod(out, M);
    write_pod(out, mult);
    write_pod(out, ef_construction);
    out.write(level0, (std::streamsize)(n * per_elem));
    for (size_t i = 0; i < n; ++i) {
        const unsigned sz = levels[i] > 0 ? (unsigned)(links * levels[i]) : 0u;
        write_pod(out, sz);
        if (sz) out.write(link_lists[i], sz);
    }
    if (!out) throw io_error(output_path);
    free(level0);
    for (char *p : link_lists) free(p);
    return 0;
}

int run(int argc, char **argv) {
    const char *tool = kToolNames[KCNA_CLI];
    Args a = parse(argc, argv);
    KGraph::IndexParams params;
    std::string data_path, output_path, res_path;
    unsigned D = 0, skip = 0, gap = 0, synthetic = 0;
    float noise = 0;
    if (a.has("data")) data_path = a.v["data"];
    if (a.has("output")) output_path = a.v["output"];
    if (a.has("result")) res_path = a.v["result"];
    get(a, "K", params.K);
    get(a, "nthreads", params.nthreads);
    get(a, "controls", params.controls);
    get(a, "nsg_R", params.nsg_R);
    get(a, "loop_i", params.loop_i);
    get(a, "search_L", params.search_L);
    get(a, "search_K", params.search_K);
    get(a, "massq_S", params.massq_S);
    get(a, "angle", params.angle);
    get(a, "step", params.step);
    get(a, "tau", params.tau);
    get(a, "iterations", params.iterations);
    get(a, "S", params.S);
    get(a, "R", params.R);
    get(a, "L", params.L);
    get(a, "delta", params.delta);
    get(a, "recall", params.recall);
    get(a, "prune", params.prune);
    get(a, "reverse", params.reverse);
    get(a, "noise", noise);
    get(a, "seed", params.seed);
    get(a, "dim", D);
    get(a, "skip", skip);
    get(a, "gap", gap);
    get(a, "synthetic", synthetic);
    get(a, "learned", params.learned_seed);
    if (a.has("screen")) {
        const std::string s = a.v["screen"];
        if (s == "fp32" || s == "0")
            params.screen = 0;
        else if (s == "bf16" || s == "1")
            params.screen = 1;
        else
            throw invalid_argument("--screen must be fp32 or bf16");
    }
    if (a.has("refine")) {
        const std::string s = a.v["refine"];
        if (s == "bridge" || s == "0")
            params.refine = 0;
        else if (s == "pool" || s == "1")
            params.refine = 1;
        else
            throw invalid_argument("--refine must be bridge or pool");
    }
    if (a.has("device")) setenv("KCNA_DEVICE", a.v["device"].c_str(), 1);
    const bool lshkit = !a.has("raw");
    if (a.has("version")) {
        printf("KGraph version %s\n", KGraph::version());
        return 0;
    }
    if (a.has("help") || (synthetic && (!a.has("dim") || a.has("data"))) ||
        (!synthetic && (!a.has("data") || (!a.has("dim") && !lshkit)))) {
        usage(tool);
        return 0;
    }
    if (params.S == 0) params.S = params.K;
    if (a.has("print-params")) {
        print_params(params, data_path, output_path, res_path);
        return 0;
    }
    if (noise != 0)
        throw invalid_argument("--noise is not supported (the reference draws it from Boost's ranlux64_base_01)");
    if (lshkit && !synthetic) {
        D = Matrix<float>::lshkit_dim(data_path);
        skip = 12;
        gap = 0;
    }
    const bool hnsw = KCNA_CLI >= 4;
    Matrix<float> data;
    std::vector<int> labels, points_num;
    double level_secs = 0;
    if (synthetic) {
        data.resize(synthetic, D);
        data.zero();
        std::default_random_engine rng(params.seed);
        std::uniform_real_distribution<double> u(-1.0, 1.0);
        for (unsigned i = 0; i < synthetic; ++i)
            for (unsigned j = 0; j < D; ++j) data[i][j] = (float)u(rng);
        if (hnsw) {
            std::vector<int> lv;
            hnsw_levels(synthetic, params.nsg_R, params.seed, lv, labels, points_num);
            // synthetic rows are i.i.d.: storage order = level order, labels map back
        }
    } else if (hnsw) {
        level_secs = data.hnsw_dataload(data_path, D, skip, gap, labels, points_num, params.nsg_R, params.seed);
    } else {
        data.load(data_path, D, skip, gap);
    }
    if (a.has("l2norm")) data.normalize2();
    printf("Size1: %u\n", data.size());
    if (hnsw) {
        if (KCNA_CLI == 5) points_num.assign(1, (int)data.size()); // fastnsw: one level
        run_hnsw(params, data, labels, points_num, level_secs, output_path, res_path);
    } else {
        MatrixOracle<Matrix<float>, metric::l2sqr> oracle(data);
        KGraph::IndexInfo info;
        KGraph *kg = KGraph::create();
        if (KCNA_CLI == 2)
            kg->buildFastTauMNG(oracle, params, &info, output_path.c_str(), res_path.c_str());
        else if (KCNA_CLI == 3)
            kg->buildFastAlphaPG(oracle, params, &info, output_path.c_str(), res_path.c_str());
        else
            kg->buildFastNSG(oracle, params, &info, output_path.c_str(), res_path.c_str());
        delete kg;
    }
    printf("%s peakmemory: %ld\n", tool, peak_memory_mb());
    return 0;
}

} // namespace

int main(int argc, char **argv) {
    try {
        return run(argc, argv);
    } catch (const std::exception &e) {
        fprintf(stderr, "%s: %s\n", kToolNames[KCNA_CLI], e.what());
        return 1;
    }
}
