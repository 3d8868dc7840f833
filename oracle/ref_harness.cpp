/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's OWN sampler code (random_walk/*.h, the app functors in
 * random_walk/apps/*.cpp and the static table initialisation of
 * creeper.h:102-175) with the counter-based Philox shim in ref_shim/SFMT.h,
 * so its outputs pin the oracle restatement.  It is compiled straight from
 * the reference sources by oracle/build_oracle.py (one binary per app,
 * TRW_REF_APP selects which app file is included) into oracle/_ref/, and is
 * only used in the container that holds the reference tree, to generate the
 * committed golden fixtures.
 *
 * The harness drives the non-interleaved *_move functions on a ring with one
 * occupied slot (every other slot empty_), setting the shim cursor
 * (walker, step = length_) before each move, then applies the update of
 * creeper.h:303-319.  The non-interleaved moves do the same sampling
 * arithmetic as the interleaved ones (same draws, same order).
 *
 * usage: ref_<app> DIR mode sampler length path_cap seed id_base p q tp [schema...]
 * DIR holds row.bin (int64 n+1), adj.bin (int32 e), sources.bin (int32 W) and
 * optionally weight.bin (double e), label.bin (int32 e).  Outputs written to
 * DIR: paths.bin, lengths.bin, steps.txt, counts.bin, and the static tables
 * alias.bin / prefix.bin / rejw.bin / rejmax.bin when mode is Static.
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#define main trw_reference_app_main
#if TRW_REF_APP == 0
#include "apps/deepwalk.cpp"
#elif TRW_REF_APP == 1
#include "apps/ppr.cpp"
#elif TRW_REF_APP == 2
#include "apps/node2vec.cpp"
#elif TRW_REF_APP == 3
#include "apps/metapath.cpp"
#else
#include "apps/genericwalk.cpp"
#endif
#undef main

namespace {

template <class T> std::vector<T> read_file(const std::string &path, bool required) {
    std::vector<T> out;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        if (required) { std::fprintf(stderr, "missing %s\n", path.c_str()); std::exit(2); }
        return out;
    }
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(sz / sizeof(T));
    if (sz && std::fread(out.data(), 1, sz, f) != (size_t)sz) std::exit(3);
    std::fclose(f);
    return out;
}

template <class T> void write_file(const std::string &path, const T *p, size_t n) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) std::exit(4);
    if (n) std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 11) { std::fprintf(stderr, "bad args\n"); return 1; }
    std::string dir = argv[1];
    int mode = std::atoi(argv[2]), sampler = std::atoi(argv[3]);
    int length = std::atoi(argv[4]), path_cap = std::atoi(argv[5]);
    uint64_t seed = std::strtoull(argv[6], nullptr, 10);
    int64_t id_base = std::strtoll(argv[7], nullptr, 10);
    double p = std::atof(argv[8]), q = std::atof(argv[9]), tp = std::atof(argv[10]);
    std::vector<int> schema;
    for (int i = 11; i < argc; ++i) schema.push_back(std::atoi(argv[i]));

    auto row = read_file<int64_t>(dir + "/row.bin", true);
    auto adj = read_file<int32_t>(dir + "/adj.bin", true);
    auto src = read_file<int32_t>(dir + "/sources.bin", true);
    auto wgt = read_file<double>(dir + "/weight.bin", false);
    auto lab = read_file<int32_t>(dir + "/label.bin", false);

    /* Populate the reference Graph (graph.h:19-83) the way load_csr does
     * (graph.cpp:45-101): offsets, adjacency (+16 padding), degrees, the
     * offset pairs (graph.cpp:86-91) and max degree (graph.cpp:590-593). */
    Graph graph;
    graph.num_vertices_ = (intT)(row.size() - 1);
    graph.num_edges_ = (int64_t)adj.size();
    graph.offset_ = new int64_t[row.size()];
    graph.degree_ = new intT[graph.num_vertices_];
    graph.offset_pair_ = new std::pair<int64_t, int64_t>[graph.num_vertices_];
    graph.adj_ = new intT[adj.size() + 16];
    graph.max_degree_ = 0;
    for (size_t i = 0; i < row.size(); ++i) graph.offset_[i] = row[i];
    for (intT v = 0; v < graph.num_vertices_; ++v) {
        graph.degree_[v] = (intT)(row[v + 1] - row[v]);
        graph.offset_pair_[v] = {row[v], row[v + 1]};
        if (graph.degree_[v] > graph.max_degree_) { graph.max_degree_ = graph.degree_[v]; graph.node_with_max_degree_ = v; }
    }
    for (size_t i = 0; i < adj.size(); ++i) graph.adj_[i] = adj[i];
    if (!wgt.empty()) {
        graph.is_edge_weighted_ = true;
        graph.edge_weight_ = new double[wgt.size() + 16];
        for (size_t i = 0; i < wgt.size(); ++i) graph.edge_weight_[i] = wgt[i];
    }
    if (!lab.empty()) {
        graph.is_edge_labeled_ = true;
        graph.edge_label_ = new int[lab.size() + 16];
        for (size_t i = 0; i < lab.size(); ++i) graph.edge_label_[i] = lab[i];
    }

    g_para.execution_ = static_cast<ExecutionMode>(mode);
    g_para.sample_ = static_cast<SamplingMethod>(sampler);
    g_para.length_ = path_cap;

#if TRW_REF_APP == 0
    DeepWalk f(length, &graph);
#elif TRW_REF_APP == 1
    PPR f(tp);
#elif TRW_REF_APP == 2
    Node2Vec f(length, 1.0 / p, 1.0 / q, &graph);  /* execute() inverts p, q (node2vec.cpp:227,234) */
#elif TRW_REF_APP == 3
    MetaPath f(length, (int)schema.size(), schema.data(), &graph);
#else
    GenericWalk f(length, &graph);
#endif
    (void)p; (void)q; (void)tp;

    if (mode == Static) {
        static_initialization(&graph, f);
        const size_t E = adj.size(), N = graph.num_vertices_;
        if (sampler == AliasSampling) write_file(dir + "/alias.bin", graph.edge_weight_alias_table_, E);
        if (sampler == InverseTransformationSampling) write_file(dir + "/prefix.bin", graph.edge_weight_prefix_sum_, E);
        if (sampler == RejectionSampling) {
            write_file(dir + "/rejw.bin", graph.edge_weight_rejection_, E);
            write_file(dir + "/rejmax.bin", graph.edge_weight_rejection_max_, N);
        }
    }

    const size_t W = src.size();
    const size_t cap = path_cap > 0 ? (size_t)path_cap : 1;
    std::vector<int32_t> paths(W * cap, -1), lengths(W, 0);
    std::vector<int32_t> counts((size_t)graph.num_vertices_, 0);
    std::vector<double> wbuf(graph.max_degree_ + 1);
    std::vector<AliasSlot> abuf(graph.max_degree_ + 1);
    std::vector<intT> seq(cap);
    std::queue<intT> large, small;
    uint64_t steps = 0;
    sfmt_t sfmt;
    sfmt_init_gen_rand(&sfmt, (uint32_t)seed);
    sfmt.seed = seed;

    for (size_t i = 0; i < W; ++i) {
        const uint64_t wid = (uint64_t)(id_base + (int64_t)i);
        BufferSlot ring[RING_SIZE];
        for (int k = 0; k < RING_SIZE; ++k) ring[k].empty_ = true;
        BufferSlot &s = ring[0];
        /* admission, creeper.h:322-331 */
        s.empty_ = false;
        s.local_id_ = 0;
        s.seq_ = seq.data();
        s.w_ = {(int)i, src[i], src[i], 1, seq.data()};
        s.seq_[0] = src[i];
        s.weight_ = wbuf.data();
        s.alias_ = abuf.data();
        for (;;) {
            sfmt.walker = wid; sfmt.step = (uint32_t)s.w_.length_; sfmt.draw = 0; sfmt.block_base = 0;
            if (mode == Uniform) {
                uniform_move(&graph, ring, &sfmt, g_para.length_);
            } else if (mode == Static) {
                if (sampler == AliasSampling) static_alias_move(&graph, ring, &sfmt, g_para.length_);
                else if (sampler == InverseTransformationSampling) static_its_move(&graph, ring, &sfmt, g_para.length_);
                else static_rs_move(&graph, ring, &sfmt, g_para.length_);
            } else if (sampler == MaxWeightRejectionSampling) {
                s.dr_ = f.max_weight(s.w_);  /* creeper.h:648-653 */
                dynamic_max_weight_rs_move(&graph, ring, &sfmt, g_para.length_, f);
            } else {
                int completed = 0, terminated = 0;
                dynamic_gather(&graph, ring, f, g_para, completed, terminated, large, small);
                if (s.empty_) break;  /* zero total weight: the walker stops (creeper.h:267-292) */
                if (sampler == InverseTransformationSampling) dynamic_its_move(&graph, ring, &sfmt, g_para.length_);
                else if (sampler == AliasSampling) dynamic_alias_move(&graph, ring, &sfmt, g_para.length_);
                else dynamic_rs_move(&graph, ring, &sfmt, g_para.length_);
            }
            /* update, creeper.h:303-319 */
            steps += 1;
            counts[s.w_.current_] += 1;
#if TRW_REF_APP == 1
            f.sfmt_.seed = seed; f.sfmt_.walker = wid; f.sfmt_.step = (uint32_t)s.w_.length_;
            f.sfmt_.draw = 0; f.sfmt_.block_base = 0x80000000u;
#endif
            if (f.update(s.w_, s.prev_, s.w_.current_, 0)) break;
        }
        lengths[i] = s.w_.length_;
        for (int k = 0; k < (int)cap && k < s.w_.length_; ++k) paths[i * cap + k] = seq[k];
    }

    write_file(dir + "/paths.bin", paths.data(), paths.size());
    write_file(dir + "/lengths.bin", lengths.data(), lengths.size());
    write_file(dir + "/counts.bin", counts.data(), counts.size());
    FILE *f_steps = std::fopen((dir + "/steps.txt").c_str(), "w");
    std::fprintf(f_steps, "%llu\n", (unsigned long long)steps);
    std::fclose(f_steps);
    return 0;
}
