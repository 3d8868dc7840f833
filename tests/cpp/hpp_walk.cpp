// Drives the C++ mirror of the reference interface (include/trw.hpp) the way
// a ThunderRW app's execute() would: load the reference's CSR files, generate
// walkers, compute<App>.  Prints steps and a checksum of every path.  A third
// argument "prebuilt" builds the graph's lookup structures before the walk.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "trw.hpp"

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    const std::string dir = argv[1];
    const std::string app = argv[2];
    trw::Graph graph = trw::Graph::load_csr(dir, /*edge_weight=*/true, /*edge_label=*/true);
    if (argc > 3 && std::string(argv[3]) == "prebuilt") graph.build_indexes();  // before the first walk
    std::vector<trw::WalkerMeta> walkers;
    trw::generate_all_source(graph, walkers, /*shuffle=*/false);
    trw::Result r;
    if (app == "deepwalk") r = trw::compute(graph, walkers, trw::DeepWalk(20));
    else if (app == "node2vec") r = trw::compute(graph, walkers, trw::Node2Vec(20, 2.0, 0.5));
    else if (app == "metapath") r = trw::compute(graph, walkers, trw::MetaPath(20, {0, 1, 2, 3, 4}));
    else if (app == "ppr") r = trw::compute(graph, walkers, trw::PPR(0.2));
    else return 3;
    unsigned long long h = 1469598103934665603ull;
    for (int32_t x : r.paths) h = (h ^ (uint32_t)x) * 1099511628211ull;
    for (int32_t x : r.lengths) h = (h ^ (uint32_t)x) * 1099511628211ull;
    std::printf("%llu %llu\n", (unsigned long long)r.steps, h);
    return 0;
}
