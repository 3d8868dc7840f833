// trw_app.cpp -- the reference's app executables over the GPU engine.
//
// ThunderRW builds one program per app (deepwalk, ppr, node2vec, metapath,
// genericwalk): creeper_main.h:14-72 parses the graph flags and loads the CSR,
// then the app's execute() parses its own flags, generates the walkers and
// calls compute<F>.  This file is compiled once per app (TRW_CLI_APP = the
// trw_app value) into thunderrw_gb300/bin/<app>, with the same flags, the same
// defaults and the same summary lines, over include/trw.hpp.
//
// Graph flags: -f <dir> (required), -ew, -el (load edge weights / labels),
// -n <threads> (accepted; the walk runs on the GPU), -vl -vw (accepted),
// -ep -al -rj (the precomputed edge-weight tables are read and installed, and
// a static walk with edge weights then uses them instead of building its
// own; the reference reads them and rebuilds, creeper.h:107-108, which for
// files written by its preprocessors gives the same tables).
// App flags (defaults as in each execute()):
//   deepwalk    -l 80 -em 1 -sm 2                (deepwalk.cpp:32-70)
//   ppr         -sp 0.2 -nw |V| -em 0 -sm 0      (ppr.cpp:36-88)
//   node2vec    -l 80 -p 2 -q 0.5 -em 2 -sm 4    (node2vec.cpp:49-103)
//   metapath    -l 80 -s <schema,...> -em 2 -sm 1 (metapath.cpp:40-104)
//   genericwalk -l 80 -st 0 -wn |V| -em 1 -sm 1  (genericwalk.cpp:32-99)
// Additions: -seed <u64> (Philox key, default 1), -o <prefix> (writes
// <prefix>.paths.bin, int32 [walkers][path_cap] padded with -1, and
// <prefix>.lengths.bin, int32 [walkers]).
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "trw.hpp"

#ifndef TRW_CLI_APP
#error "compile with -DTRW_CLI_APP=<trw_app value>"
#endif

namespace {

const char *kModes[] = {"Uniform", "Static", "Dynamic"};
const char *kSamplers[] = {"UniformSampling", "InverseTransformationSampling", "AliasSampling",
                           "RejectionSampling", "MaxWeightRejectionSampling"};
const char *kAppNames[] = {"deepwalk", "ppr", "node2vec", "metapath", "genericwalk"};

// InputParser (util/command_parser.h:12-39): a flag's value is the token after it.
struct Flags {
    std::vector<std::string> tok;
    Flags(int argc, char **argv) : tok(argv + 1, argv + argc) {}
    bool has(const char *f) const {
        for (const auto &t : tok)
            if (t == f) return true;
        return false;
    }
    std::string get(const char *f) const {
        for (size_t i = 0; i + 1 < tok.size(); ++i)
            if (tok[i] == f) return tok[i + 1];
        return "";
    }
    int get_int(const char *f, int dflt) const {
        const std::string v = get(f);
        return v.empty() ? dflt : std::stoi(v);
    }
};

void usage() {
    std::fprintf(stderr,
                 "usage: %s -f <graph dir> [-ew] [-el] [-n threads] [-seed S] [-o prefix] <app flags>\n"
                 "app flags: deepwalk -l -em -sm | ppr -sp -nw -em -sm | node2vec -l -p -q -em -sm |\n"
                 "           metapath -l -s a,b,c -em -sm | genericwalk -l -st -wn -em -sm\n",
                 kAppNames[TRW_CLI_APP]);
}

void log_info(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
void log_info(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::fputs("[info] ", stdout);
    std::vprintf(fmt, ap);
    std::fputc('\n', stdout);
    va_end(ap);
}

bool write_file(const std::string &path, const void *data, size_t bytes) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}

// generate_single_source (walker_generator.cpp:42-63) also reports the hub.
void single_source(const trw::Graph &g, std::vector<trw::WalkerMeta> &w, int count) {
    trw::generate_single_source(g, w, count);
    const int32_t u = w.empty() ? 0 : w[0].source_;
    std::printf("%d %d\n", u, g.degree(u));
}

template <class App>
int run(trw::Graph &g, std::vector<trw::WalkerMeta> &walkers, const App &app, trw::HyperParameter para,
        const Flags &fl, int threads) {
    const uint64_t seed = fl.get("-seed").empty() ? 1ull : std::stoull(fl.get("-seed"));
    log_info("Configuration: %s, %s, thread num %d, length %d, walkers %zu, seed %llu",
             kModes[para.execution_ % 3], kSamplers[para.sample_ % 5], threads, para.length_, walkers.size(),
             (unsigned long long)seed);
    // static_initialization runs before the walk timer (creeper.h:700-739)
    if (para.execution_ == trw::Static &&
        !(App::app != TRW_APP_PPR && g.table_loaded(para.sample_))) {
        const int kind = App::app == TRW_APP_PPR ? TRW_WEIGHTS_UNIT : TRW_WEIGHTS_EDGE;
        const auto t0 = std::chrono::steady_clock::now();
        trw::check(trw_tables_build(g.handle(), para.sample_, kind, nullptr));
        trw::check(trw_graph_synchronize(g.handle()));
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        log_info("Initialization time (seconds): %.6lf", s);
    }
    const auto t0 = std::chrono::steady_clock::now();
    trw::Result r = trw::compute(g, walkers, app, para, seed);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    log_info("Walking time (seconds): %.6lf", s);
    log_info("Num of steps: %llu", (unsigned long long)r.steps);
    log_info("Throughput (steps per second): %.2lf", s > 0 ? r.steps / s : 0.0);
    const std::string out = fl.get("-o");
    if (!out.empty()) {
        if (!write_file(out + ".paths.bin", r.paths.data(), r.paths.size() * sizeof(int32_t)) ||
            !write_file(out + ".lengths.bin", r.lengths.data(), r.lengths.size() * sizeof(int32_t))) {
            std::fprintf(stderr, "error: cannot write %s.paths.bin / .lengths.bin\n", out.c_str());
            return 1;
        }
        log_info("Paths written to %s.paths.bin ([%zu][%d] int32)", out.c_str(), walkers.size(), r.path_cap);
    }
    return 0;
}

trw::HyperParameter para(const Flags &fl, int em, int sm, int length) {
    return {static_cast<trw::ExecutionMode>(fl.get_int("-em", em)),
            static_cast<trw::SamplingMethod>(fl.get_int("-sm", sm)), length};
}

int execute(trw::Graph &g, const Flags &fl, int threads) {
    std::vector<trw::WalkerMeta> walkers;
    const int l = fl.get_int("-l", 80);
    switch (TRW_CLI_APP) {
    case TRW_APP_DEEPWALK: {
        trw::generate_all_source(g, walkers);
        return run(g, walkers, trw::DeepWalk(l), para(fl, trw::Static, trw::AliasSampling, l), fl, threads);
    }
    case TRW_APP_PPR: {
        const double sp = fl.get("-sp").empty() ? 0.2 : std::stod(fl.get("-sp"));
        const int nw = fl.get_int("-nw", g.num_vertices());
        single_source(g, walkers, nw);
        std::printf("%d\n", walkers.empty() ? -1 : walkers[0].source_);
        return run(g, walkers, trw::PPR(sp), para(fl, trw::Uniform, trw::UniformSampling, 1), fl, threads);
    }
    case TRW_APP_NODE2VEC: {
        // parsed as float, as node2vec.cpp:64-75 does with std::stof
        const double p = fl.get("-p").empty() ? 2.0 : (double)std::stof(fl.get("-p"));
        const double q = fl.get("-q").empty() ? 0.5 : (double)std::stof(fl.get("-q"));
        trw::generate_all_source(g, walkers);
        return run(g, walkers, trw::Node2Vec(l, p, q), para(fl, trw::Dynamic, trw::MaxWeightRejectionSampling, l),
                   fl, threads);
    }
    case TRW_APP_METAPATH: {
        const std::string s = fl.get("-s");
        if (s.empty()) {
            std::fprintf(stderr, "error: metapath needs -s <schema>, e.g. -s 0,1,2\n");
            return 2;
        }
        std::vector<int32_t> schema;
        size_t at = 0;
        while (at <= s.size()) {
            const size_t comma = s.find(',', at);
            const std::string t = s.substr(at, comma == std::string::npos ? std::string::npos : comma - at);
            if (!t.empty()) schema.push_back(std::stoi(t));
            if (comma == std::string::npos) break;
            at = comma + 1;
        }
        for (int32_t x : schema) std::printf("%d ", x);
        std::printf("\n");
        trw::generate_all_source(g, walkers);
        return run(g, walkers, trw::MetaPath(l, schema),
                   para(fl, trw::Dynamic, trw::InverseTransformationSampling, l), fl, threads);
    }
    default: {
        const int st = fl.get_int("-st", 0);  // SourceType: 0 all, 1 single, 2 random
        int wn = fl.get_int("-wn", g.num_vertices());
        if (wn == 0) wn = g.num_vertices();
        if (st == 0) trw::generate_all_source(g, walkers);
        else if (st == 1) single_source(g, walkers, wn);
        else trw::generate_random_source(g, walkers, wn, 0);
        return run(g, walkers, trw::GenericWalk(l), para(fl, trw::Static, trw::InverseTransformationSampling, l),
                   fl, threads);
    }
    }
}

}  // namespace

int main(int argc, char **argv) {
    Flags fl(argc, argv);
    if (fl.has("-h") || fl.has("--help")) {
        usage();
        return 0;
    }
    const std::string dir = fl.get("-f");
    if (dir.empty()) {
        usage();
        return 2;
    }
    try {
        const int threads = fl.get_int("-n", 1);
        trw::Graph g = trw::Graph::load_csr(dir, fl.has("-ew"), fl.has("-el"));
        log_info("Graph: |V| = %d, |E| = %lld, max degree = %d, %s, %s", g.num_vertices(),
                 (long long)g.num_edges(), g.max_degree(), fl.has("-ew") ? "edge weighted" : "edge unweighted",
                 fl.has("-el") ? "edge labeled" : "edge unlabeled");
        if (fl.has("-ep") || fl.has("-al") || fl.has("-rj")) {
            g.load_tables(dir, fl.has("-ep"), fl.has("-al"), fl.has("-rj"));
            log_info("Loaded tables:%s%s%s", fl.has("-ep") ? " prefix sums" : "", fl.has("-al") ? " alias" : "",
                     fl.has("-rj") ? " rejection maxima" : "");
        }
        const int rc = execute(g, fl, threads);
        if (rc == 0) log_info("Done.");
        return rc;
    } catch (const trw::Error &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 2;
    }
}
