// trw_build.cu -- device table builders and CSR validation.
//
// The reference builds its sampling tables per vertex with sequential double
// arithmetic (static_initialization, creeper.h:102-175; the offline
// alias_preprocess.cpp:30-73, its_preprocess.cpp:21-34,
// rejection_preprocess.cpp:24-27).  Bit-identical tables need the same
// operation order, so every vertex's arithmetic chain stays sequential in one
// thread; the parallelism is across vertices.  The maximum is
// order-independent and uses the same per-vertex loop for simplicity.
#include "trw_device.cuh"
#include "trw_internal.h"

namespace trw {
namespace {

__device__ __forceinline__ double sweight(const DevGraph &g, int unit, int64_t eid) {
    return unit ? 1.0 : __ldg(g.weight + eid);
}

// alias_initialization (alias_sampling.h:12-54) for one vertex, written into
// its own table rows with no other scratch.
//
// The small queue of the reference holds the initial smalls (index order)
// followed by the larges in the order they turn small, and larges turn small
// strictly in index order (only the front large changes).  So pop number j
// of the pairing loop pops the j-th entry of the stable small-then-large
// partition P, writes table slot j, and the leftover loops continue with
// slots j+1.. in the same order.  Slot j therefore holds P[j] (in .first)
// until it is written; a large that turns small parks its final value in its
// own slot, which is written exactly when it is popped.
__global__ void build_alias_kernel(const DevGraph g, int unit, AliasSlot *out) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.n) return;
    const int2 r = __ldg(g.rows + v);
    const int32_t d = r.y - r.x;
    if (d <= 0) return;
    const int32_t *nb = g.adj + r.x;
    AliasSlot *tab = out + r.x;
    double sum = 0.0;
    for (int32_t j = 0; j < d; ++j) sum += sweight(g, unit, r.x + j);  // std::accumulate
    const double avg = sum / d;
    if (avg == 0.0) {
        // all-zero row: the reference leaves these slots uninitialised; here
        // every neighbour is equally likely
        for (int32_t j = 0; j < d; ++j) { const int32_t x = __ldg(nb + j); tab[j] = {1.0, x, x}; }
        return;
    }
    int32_t ns = 0;
    for (int32_t j = 0; j < d; ++j) ns += (sweight(g, unit, r.x + j) / avg) < 1;
    int32_t si = 0, li = ns;
    for (int32_t j = 0; j < d; ++j) {
        const double sc = sweight(g, unit, r.x + j) / avg;  // src[j] /= weight_avg
        const int32_t pos = sc < 1 ? si++ : li++;
        tab[pos].prob = sc;
        tab[pos].first = j;
    }
    const int32_t nl = d - ns;
    int32_t sp = 0, c = 0;
    double vl = nl ? tab[ns].prob : 0.0;
    while (sp < ns + c && c < nl) {
        const double vs = tab[sp].prob;
        const int32_t s_idx = tab[sp].first;
        const int32_t l_idx = tab[ns + c].first;
        tab[sp].first = __ldg(nb + s_idx);
        tab[sp].second = __ldg(nb + l_idx);
        ++sp;
        vl = vl + vs - 1;  // src[large] + src[small] - 1
        if (vl < 1) {
            tab[ns + c].prob = vl;
            ++c;
            if (c < nl) vl = tab[ns + c].prob;
        }
    }
    for (int32_t j = sp; j < d; ++j) {
        const int32_t x = __ldg(nb + tab[j].first);
        tab[j].prob = 1.0;
        tab[j].first = x;
        tab[j].second = x;
    }
}

// its_initialization (inverse_transformation_sampling.h:19-24).
__global__ void build_prefix_kernel(const DevGraph g, int unit, double *out) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.n) return;
    const int2 r = __ldg(g.rows + v);
    if (r.y <= r.x) return;
    double acc = sweight(g, unit, r.x);
    out[r.x] = acc;
    for (int32_t i = r.x + 1; i < r.y; ++i) {
        acc = acc + sweight(g, unit, i);
        out[i] = acc;
    }
}

// rs_initialization (rejection_sampling.h:12-14): *max_element.
__global__ void build_max_kernel(const DevGraph g, int unit, double *out) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.n) return;
    const int2 r = __ldg(g.rows + v);
    double mx = 0.0;
    for (int32_t i = r.x; i < r.y; ++i) {
        const double w = sweight(g, unit, i);
        mx = (i == r.x || w > mx) ? w : mx;  // first maximum, as std::max_element
    }
    out[v] = mx;
}

// CSR validation: offsets start at 0, end at e and never decrease; every
// neighbour id is in range; optionally every row is sorted ascending
// (Graph::is_sort, graph.cpp:764-776).  Also packs the (begin, end) pairs.
__global__ void validate_kernel(const int64_t *row, const int32_t *adj, int32_t n, int64_t e, int check_sorted,
                                int2 *rows_out, int *bad, int *max_degree) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int64_t b = row[v], en = row[v + 1];
    if (v == 0 && b != 0) atomicOr(bad, 1);
    if (v == n - 1 && en != e) atomicOr(bad, 1);
    if (b < 0 || en < b || en > e) { atomicOr(bad, 2); return; }
    rows_out[v] = make_int2((int32_t)b, (int32_t)en);
    atomicMax(max_degree, (int)(en - b));
    int32_t last = -1;
    for (int64_t i = b; i < en; ++i) {
        const int32_t x = adj[i];
        if (x < 0 || x >= n) { atomicOr(bad, 4); return; }
        if (check_sorted && x < last) { atomicOr(bad, 8); return; }
        last = x;
    }
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

cudaError_t launch_build_alias(const DevGraph &g, int unit, AliasSlot *out, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_alias_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    return cudaGetLastError();
}

cudaError_t launch_build_prefix(const DevGraph &g, int unit, double *out, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_prefix_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    return cudaGetLastError();
}

cudaError_t launch_build_max(const DevGraph &g, int unit, double *out, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_max_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    return cudaGetLastError();
}

cudaError_t launch_validate_graph(const int64_t *row, const int32_t *adj, int32_t n, int64_t e, int check_sorted,
                                  int2 *rows_out, int *bad, int *max_degree, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    validate_kernel<<<blocks_for(n), 256, 0, st>>>(row, adj, n, e, check_sorted, rows_out, bad, max_degree);
    return cudaGetLastError();
}

}  // namespace trw
