// trw.hpp -- C++ host mirror of ThunderRW's walk interface over the C ABI.
//
// The reference is used as (random_walk/apps/deepwalk.cpp:32-70):
//
//     Graph graph; graph.is_edge_weighted_ = true; graph.load_csr(dir);
//     g_para.length_ = 80;  // + execution_, sample_
//     std::vector<WalkerMeta> walkers; generate_all_source(graph, walkers);
//     compute(graph, walkers, DeepWalk(80, &graph));
//
// With this header the same program reads:
//
//     trw::Graph graph = trw::Graph::load_csr(dir, /*edge_weight=*/true);
//     std::vector<trw::WalkerMeta> walkers; trw::generate_all_source(graph, walkers);
//     trw::Result r = trw::compute(graph, walkers, trw::DeepWalk(80));
//
// The app structs carry the functor's constructor arguments and its g_para
// defaults; their weight / update / max_weight hooks run as device twins in
// libtrw_gpu.so.  Errors throw trw::Error (the reference asserts or exits).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <memory>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "trw.h"

namespace trw {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != TRW_OK) throw Error(rc, trw_last_error());
}

// ExecutionMode / SamplingMethod (types.h:41-59) and HyperParameter (types.h:72-77).
enum ExecutionMode { Uniform = TRW_MODE_UNIFORM, Static = TRW_MODE_STATIC, Dynamic = TRW_MODE_DYNAMIC };
enum SamplingMethod {
    UniformSampling = TRW_SAMPLER_UNIFORM,
    InverseTransformationSampling = TRW_SAMPLER_ITS,
    AliasSampling = TRW_SAMPLER_ALIAS,
    RejectionSampling = TRW_SAMPLER_REJECTION,
    MaxWeightRejectionSampling = TRW_SAMPLER_MAXWEIGHT_REJECTION
};
struct HyperParameter {
    ExecutionMode execution_;
    SamplingMethod sample_;
    int length_;  // path entries recorded per walker (g_para.length_)
};

// WalkerMeta (walker.h:9-15).  seq_ points into the Result's path buffer.
struct WalkerMeta {
    int id_;
    int source_;
    int current_;
    int length_;
    int *seq_;
};

// The reference's app functors (apps/*.cpp) with their g_para defaults.
struct DeepWalk {
    int l_;
    explicit DeepWalk(int l = 80) : l_(l) {}
    static constexpr int app = TRW_APP_DEEPWALK;
    HyperParameter defaults() const { return {Static, AliasSampling, l_}; }       // deepwalk.cpp:7,37-56
    void fill(trw_walk_desc &d) const { d.length = l_; }
};
struct PPR {
    double tp_;
    explicit PPR(double tp = 0.2) : tp_(tp) {}
    static constexpr int app = TRW_APP_PPR;
    HyperParameter defaults() const { return {Uniform, UniformSampling, 1}; }     // ppr.cpp:80,123
    void fill(trw_walk_desc &d) const { d.tp = tp_; d.length = 1; }
};
struct Node2Vec {
    int l_;
    double p_, q_;  // the user-facing parameters; the hooks weigh 1/p and 1/q
    Node2Vec(int l = 80, double p = 2.0, double q = 0.5) : l_(l), p_(p), q_(q) {}
    static constexpr int app = TRW_APP_NODE2VEC;
    HyperParameter defaults() const { return {Dynamic, MaxWeightRejectionSampling, l_}; }  // node2vec.cpp:165
    void fill(trw_walk_desc &d) const { d.length = l_; d.p = p_; d.q = q_; }
};
struct MetaPath {
    int l_;
    std::vector<int32_t> schema_;
    MetaPath(int l, std::vector<int32_t> schema) : l_(l), schema_(std::move(schema)) {}
    static constexpr int app = TRW_APP_METAPATH;
    HyperParameter defaults() const { return {Dynamic, InverseTransformationSampling, l_}; }  // metapath.cpp:7
    void fill(trw_walk_desc &d) const {
        d.length = l_;
        d.schema = schema_.data();
        d.schema_len = (int32_t)schema_.size();
    }
};
struct GenericWalk {
    int l_;
    explicit GenericWalk(int l = 80) : l_(l) {}
    static constexpr int app = TRW_APP_GENERICWALK;
    HyperParameter defaults() const { return {Static, AliasSampling, l_}; }       // genericwalk.cpp:110
    void fill(trw_walk_desc &d) const { d.length = l_; }
};

// Graph (graph.h:19-329): the CSR lives in HBM; host copies of the degree
// array are kept for the walker generators.
class Graph {
public:
    Graph(const int64_t *offset, const int32_t *adj, const double *weight, const int32_t *label, int32_t n,
          int64_t e, bool check_sorted = false)
        : degree_(n) {
        trw_graph *h = nullptr;
        check(trw_graph_create(offset, adj, weight, label, n, e, check_sorted ? TRW_GRAPH_CHECK_SORTED : 0u, &h));
        h_.reset(h, [](trw_graph *p) { trw_graph_destroy(p); });
        int32_t md = 0;
        check(trw_graph_info(h, &n_, &e_, &md));
        max_degree_ = md;
        for (int32_t v = 0; v < n; ++v) degree_[v] = (int32_t)(offset[v + 1] - offset[v]);
    }

    // Graph::load_csr (graph.cpp:45-101) over the reference's files.
    static Graph load_csr(const std::string &dir, bool edge_weight = false, bool edge_label = false) {
        std::ifstream df(dir + "/b_degree.bin", std::ios::binary);
        if (!df) throw Error(TRW_ERR_INVALID, "cannot open " + dir + "/b_degree.bin");
        uint32_t elem = 0;
        int32_t n = 0;
        int64_t e = 0;
        df.read(reinterpret_cast<char *>(&elem), 4);
        df.read(reinterpret_cast<char *>(&n), 4);
        df.read(reinterpret_cast<char *>(&e), 8);
        if (elem != 4 || n <= 0 || e < 0) throw Error(TRW_ERR_INVALID, "bad b_degree.bin header");
        std::vector<int32_t> deg(n);
        df.read(reinterpret_cast<char *>(deg.data()), 4 * (std::streamsize)n);
        std::vector<int64_t> off(n + 1, 0);
        for (int32_t v = 0; v < n; ++v) off[v + 1] = off[v] + deg[v];
        if (off[n] != e) throw Error(TRW_ERR_INVALID, "degree sum differs from e");
        auto slurp = [&](const std::string &name, void *dst, size_t bytes) {
            std::ifstream f(dir + "/" + name, std::ios::binary);
            if (!f || !f.read(static_cast<char *>(dst), (std::streamsize)bytes))
                throw Error(TRW_ERR_INVALID, "cannot read " + dir + "/" + name);
        };
        std::vector<int32_t> adj(e), lab;
        std::vector<double> w;
        slurp("b_adj.bin", adj.data(), 4 * (size_t)e);
        if (edge_weight) { w.resize(e); slurp("b_edge_weight.bin", w.data(), 8 * (size_t)e); }
        if (edge_label) { lab.resize(e); slurp("b_edge_label.bin", lab.data(), 4 * (size_t)e); }
        return Graph(off.data(), adj.data(), edge_weight ? w.data() : nullptr, edge_label ? lab.data() : nullptr, n,
                     e);
    }

    // The precomputed sampling tables the reference loads under -ep, -al and
    // -rj (graph.cpp:78-94: b_edge_weight_prefix_sum.bin,
    // b_edge_weight_alias_table.bin, b_edge_weight_max.bin), installed as the
    // graph's edge-weight tables so that static walks do not build them.
    void load_tables(const std::string &dir, bool prefix_sum, bool alias_table, bool rejection_max) {
        auto install = [&](const char *name, int32_t sampler, size_t bytes) {
            std::vector<char> buf(bytes);
            std::ifstream f(dir + "/" + name, std::ios::binary);
            if (!f || !f.read(buf.data(), (std::streamsize)bytes))
                throw Error(TRW_ERR_INVALID, "cannot read " + dir + "/" + name);
            check(trw_tables_upload(h_.get(), sampler, TRW_WEIGHTS_EDGE, buf.data(), bytes, nullptr));
            loaded_ |= 1u << sampler;
        };
        if (prefix_sum) install("b_edge_weight_prefix_sum.bin", TRW_SAMPLER_ITS, 8 * (size_t)e_);
        if (alias_table) install("b_edge_weight_alias_table.bin", TRW_SAMPLER_ALIAS, 16 * (size_t)e_);
        if (rejection_max) install("b_edge_weight_max.bin", TRW_SAMPLER_REJECTION, 8 * (size_t)n_);
    }
    // Whether load_tables installed the edge-weight table of `sampler`.
    bool table_loaded(int32_t sampler) const { return (loaded_ >> sampler) & 1u; }

    int32_t num_vertices() const { return n_; }
    int64_t num_edges() const { return e_; }
    int32_t max_degree() const { return max_degree_; }
    int32_t degree(int32_t v) const { return degree_[v]; }
    trw_graph *handle() const { return h_.get(); }

    // Builds the Node2Vec edge set and the MetaPath label index now instead
    // of in the first walk that needs them (e.g. before timing or serving).
    void build_indexes(bool edge_set = true, bool label_index = true) {
        check(trw_graph_build_indexes(h_.get(), edge_set ? 1 : 0, label_index ? 1 : 0, nullptr));
    }

private:
    std::shared_ptr<trw_graph> h_;
    std::vector<int32_t> degree_;
    int32_t n_ = 0;
    int64_t e_ = 0;
    int32_t max_degree_ = 0;
    uint32_t loaded_ = 0;
};

// Walker generators (walker_generator.cpp:9-63).  The reference shuffles
// with std::mt19937(0) (utility.h:96-100), reproduced here with the same
// engine and std::shuffle.
inline void generate_all_source(const Graph &g, std::vector<WalkerMeta> &walkers, bool shuffle = true) {
    std::vector<int32_t> src;
    for (int32_t v = 0; v < g.num_vertices(); ++v)
        if (g.degree(v) != 0) src.push_back(v);
    if (shuffle) {
        std::mt19937 rng(0);
        std::shuffle(src.begin(), src.end(), rng);
    }
    walkers.clear();
    for (size_t i = 0; i < src.size(); ++i) walkers.push_back({(int)i, src[i], src[i], 1, nullptr});
}

inline void generate_single_source(const Graph &g, std::vector<WalkerMeta> &walkers, int count) {
    int32_t u = 0, d = g.degree(0);
    for (int32_t v = 1; v < g.num_vertices(); ++v)
        if (g.degree(v) > d) { d = g.degree(v); u = v; }
    walkers.clear();
    for (int i = 0; i < count; ++i) walkers.push_back({i, u, u, 1, nullptr});
}

// generate_random_source (walker_generator.cpp:27-40): `count` walkers from
// uniformly drawn vertices with at least one neighbour.  The reference draws
// with SFMT seeded by `seed`; this draws from the library's Philox stream
// (draw j = word j%4 of block (j/4, 0, 0xffffffff, 0xffffffff) under key
// (seed, 0)), so the sources differ from the reference's as every walk does.
inline uint32_t philox_word(uint64_t seed, uint64_t j) {
    uint32_t c[4] = {(uint32_t)(j >> 2), 0u, 0xffffffffu, 0xffffffffu};
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    }
    return c[j & 3];
}

inline void generate_random_source(const Graph &g, std::vector<WalkerMeta> &walkers, int count, uint64_t seed = 0) {
    walkers.clear();
    bool any = false;
    for (int32_t v = 0; v < g.num_vertices() && !any; ++v) any = g.degree(v) != 0;
    if (!any) return;
    for (uint64_t j = 0; (int)walkers.size() < count; ++j) {
        const int32_t u = (int32_t)(philox_word(seed, j) % (uint32_t)g.num_vertices());
        if (g.degree(u) != 0) walkers.push_back({(int)walkers.size(), u, u, 1, nullptr});
    }
}

struct Result {
    uint64_t steps = 0;
    std::vector<int32_t> paths;    // walkers x path_cap, -1 padded
    std::vector<int32_t> lengths;  // final length_ per walker
    int32_t path_cap = 0;
};

// compute<F>(graph, walkers, f) (creeper.h:689-831): walks every walker to
// completion on the GPU.  walkers[i].length_ / current_ / seq_ are updated as
// the reference's LOG_SEQUENCE build does (creeper.h:310-317).
template <class F>
Result compute(Graph &graph, std::vector<WalkerMeta> &walkers, const F &f, HyperParameter para,
               uint64_t seed = 1, trw_stream_t stream = nullptr) {
    trw_walk_desc d{};
    d.app = F::app;
    d.mode = para.execution_;
    d.sampler = para.sample_;
    d.seed = seed;
    f.fill(d);
    std::vector<int32_t> src(walkers.size());
    for (size_t i = 0; i < walkers.size(); ++i) src[i] = walkers[i].source_;
    Result r;
    r.path_cap = para.length_ > 0 ? para.length_ : 1;
    r.paths.resize(walkers.size() * (size_t)r.path_cap);
    r.lengths.resize(walkers.size());
    check(trw_walk(graph.handle(), &d, src.data(), (int64_t)src.size(), walkers.empty() ? 0 : walkers[0].id_,
                   r.paths.data(), r.path_cap, r.lengths.data(), nullptr, &r.steps, TRW_ENGINE_PERSISTENT, stream));
    for (size_t i = 0; i < walkers.size(); ++i) {
        walkers[i].length_ = r.lengths[i];
        walkers[i].seq_ = r.paths.data() + i * (size_t)r.path_cap;
        const int last = std::min(r.lengths[i], r.path_cap) - 1;
        walkers[i].current_ = walkers[i].seq_[last];
    }
    return r;
}

template <class F>
Result compute(Graph &graph, std::vector<WalkerMeta> &walkers, const F &f) {
    return compute(graph, walkers, f, f.defaults());
}

}  // namespace trw
