// trw_build.cu -- device table builders and CSR validation.
//
// The reference builds its sampling tables per vertex with sequential double
// arithmetic (static_initialization, creeper.h:102-175; the offline
// alias_preprocess.cpp:30-73, its_preprocess.cpp:21-34,
// rejection_preprocess.cpp:24-27).  Bit-identical tables need the same
// operation order, so every vertex's arithmetic chain stays sequential.
// Rows of up to kWarpRow entries are built one thread per vertex; longer rows
// (the hubs of power-law graphs) one warp per vertex, where the warp loads
// 32 entries at a time with coalesced loads and runs the sequential chains in
// lockstep through shuffles.  The maximum is order-independent.
#include <algorithm>
#include <climits>

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
constexpr int32_t kWarpRow = 32;

__global__ void build_alias_kernel(const DevGraph g, int unit, AliasSlot *out) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.n) return;
    const int2 r = __ldg(g.rows + v);
    const int32_t d = r.y - r.x;
    if (d <= 0 || d > kWarpRow) return;
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
    if (r.y <= r.x || r.y - r.x > kWarpRow) return;
    double acc = sweight(g, unit, r.x);
    out[r.x] = acc;
    for (int32_t i = r.x + 1; i < r.y; ++i) {
        acc = acc + sweight(g, unit, i);
        out[i] = acc;
    }
}

// ---- one warp per long row -------------------------------------------------

constexpr unsigned kFull = 0xffffffffu;

// Left fold of the row's weights (std::accumulate order): every lane keeps
// the same running sum, adding the 32 staged entries in order.
__device__ __forceinline__ double warp_row_sum(const DevGraph &g, int unit, int2 r) {
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int32_t base = r.x; base < r.y; base += 32) {
        const int32_t i = base + lane;
        const double w = i < r.y ? sweight(g, unit, i) : 0.0;
        const int m = min(32, r.y - base);
        for (int k = 0; k < m; ++k) acc = acc + __shfl_sync(kFull, w, k);
    }
    return acc;
}

// its_initialization for a long row: the same left-to-right chain; lane k
// keeps the value after adding entry k of the block and stores it (coalesced).
__global__ void build_prefix_warp_kernel(const DevGraph g, int unit, double *out, const int32_t *long_rows) {
    const int32_t v = long_rows[blockIdx.x];  // one warp per block: long rows spread over the SMs
    const int lane = threadIdx.x & 31;
    const int2 r = __ldg(g.rows + v);
    if (r.y - r.x <= kWarpRow) return;
    double acc = 0.0;
    bool first = true;
    for (int32_t base = r.x; base < r.y; base += 32) {
        const int32_t i = base + lane;
        const double w = i < r.y ? sweight(g, unit, i) : 0.0;
        const int m = min(32, r.y - base);
        double mine = 0.0;
        for (int k = 0; k < m; ++k) {
            const double x = __shfl_sync(kFull, w, k);
            acc = first ? x : acc + x;  // dst[0] = src[0]; dst[i] = dst[i-1] + src[i]
            first = false;
            if (lane == k) mine = acc;
        }
        if (i < r.y) out[i] = mine;
    }
}

// alias_initialization for a long row (same slot formulation as the thread
// kernel above): ballot-based stable partition, then the pairing loop run in
// lockstep by the warp with 32-entry register blocks of the small queue and
// of the large list; table entries hold neighbour indices until a final
// parallel pass maps them to vertex ids.
__global__ void build_alias_warp_kernel(const DevGraph g, int unit, AliasSlot *out, const int32_t *long_rows) {
    const int32_t v = long_rows[blockIdx.x];  // one warp per block: long rows spread over the SMs
    const int lane = threadIdx.x & 31;
    const int2 r = __ldg(g.rows + v);
    const int32_t d = r.y - r.x;
    if (d <= kWarpRow) return;
    const int32_t *nb = g.adj + r.x;
    AliasSlot *tab = out + r.x;
    const double avg = warp_row_sum(g, unit, r) / d;
    if (avg == 0.0) {
        for (int32_t j = lane; j < d; j += 32) { const int32_t x = __ldg(nb + j); tab[j] = {1.0, x, x}; }
        return;
    }
    // stable partition: smalls (w/avg < 1) first, in index order
    int32_t ns = 0;
    for (int32_t base = 0; base < d; base += 32) {
        const int32_t j = base + lane;
        ns += __popc(__ballot_sync(kFull, j < d && sweight(g, unit, r.x + j) / avg < 1));
    }
    int32_t sb = 0, lb = ns;
    for (int32_t base = 0; base < d; base += 32) {
        const int32_t j = base + lane;
        const bool in = j < d;
        const double sc = in ? sweight(g, unit, r.x + j) / avg : 0.0;
        const unsigned ms = __ballot_sync(kFull, in && sc < 1), ml = __ballot_sync(kFull, in && !(sc < 1));
        if (in) {
            const unsigned below = (1u << lane) - 1u;
            const int32_t pos = sc < 1 ? sb + __popc(ms & below) : lb + __popc(ml & below);
            tab[pos].prob = sc;
            tab[pos].first = j;
        }
        sb += __popc(ms);
        lb += __popc(ml);
    }
    __syncwarp();
    // pairing loop (alias_sampling.h:29-39) in lockstep
    const int32_t nl = d - ns;
    int32_t sp = 0, c = 0;
    int32_t sblk = -1, lblk = -1;
    double s_prob = 0.0, l_prob = 0.0;
    int32_t s_idx = 0, l_idx = 0;
    auto load_l = [&](int32_t pos) {  // large list entries are untouched until stashed
        lblk = pos;
        const int32_t j = pos + lane;
        if (j < d) { l_prob = tab[j].prob; l_idx = tab[j].first; }
    };
    if (nl) load_l(ns);
    double vl = __shfl_sync(kFull, l_prob, 0);
    while (sp < ns + c && c < nl) {
        // small queue head: slot sp.  Slots >= ns hold larges, whose value
        // changes when they turn small; the cached block is kept in step with
        // those changes below, so it is reloaded only every 32 smalls.
        if (sblk < 0 || sp >= sblk + 32) {
            __syncwarp();
            sblk = sp;
            const int32_t j = sp + lane;
            if (j < d) { s_prob = tab[j].prob; s_idx = tab[j].first; }
        }
        const double vs = __shfl_sync(kFull, s_prob, sp - sblk);
        const int32_t si = __shfl_sync(kFull, s_idx, sp - sblk);
        const int32_t li = __shfl_sync(kFull, l_idx, ns + c - lblk);
        if (lane == 0) { tab[sp].prob = vs; tab[sp].first = si; tab[sp].second = li; }
        ++sp;
        vl = vl + vs - 1;  // src[large] + src[small] - 1
        if (vl < 1) {
            if (lane == 0) tab[ns + c].prob = vl;
            if (lane == ns + c - sblk) s_prob = vl;  // the cached copy of slot ns + c, if cached
            ++c;
            if (c < nl) {
                if (ns + c >= lblk + 32) { __syncwarp(); load_l(ns + c); }
                vl = __shfl_sync(kFull, l_prob, ns + c - lblk);
            }
        }
    }
    __syncwarp();
    // indices -> vertex ids; leftovers (slots >= sp) get probability 1
    for (int32_t j = lane; j < d; j += 32) {
        AliasSlot e = tab[j];
        if (j >= sp) { e.prob = 1.0; e.second = e.first; }
        e.first = __ldg(nb + e.first);
        e.second = __ldg(nb + e.second);
        tab[j] = e;
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
// One warp per vertex reads the row with coalesced loads; each lane compares
// its entry with the previous lane's (and the previous chunk's last entry).
__global__ void validate_kernel(const int64_t *row, const int32_t *adj, int32_t n, int64_t e, int check_sorted,
                                int2 *rows_out, int *bad, int *max_degree) {
    const int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (v >= n) return;
    const int64_t b = row[v], en = row[v + 1];
    if (lane == 0) {
        if (v == 0 && b != 0) atomicOr(bad, 1);
        if (v == n - 1 && en != e) atomicOr(bad, 1);
    }
    if (b < 0 || en < b || en > e) { if (lane == 0) atomicOr(bad, 2); return; }
    if (lane == 0) {
        rows_out[v] = make_int2((int32_t)b, (int32_t)en);
        atomicMax(max_degree, (int)(en - b));
    }
    int32_t carry = -1;  // last entry of the previous chunk
    int flags = 0;
    for (int64_t base = b; base < en; base += 32) {
        const int64_t i = base + lane;
        const bool in = i < en;
        const int32_t x = in ? adj[i] : 0x7fffffff;
        if (in && (x < 0 || x >= n)) flags |= 4;
        int32_t left = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane == 0) left = carry;
        if (check_sorted && in && x < left) flags |= 8;
        carry = __shfl_sync(0xffffffffu, x, 31);
    }
    flags = __reduce_or_sync(0xffffffffu, flags);
    if (lane == 0 && flags) atomicOr(bad, flags);
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }

// (degree, vertex) of every row longer than kWarpRow, appended in any order.
__global__ void collect_long_rows_kernel(const DevGraph g, int2 *list, int *count) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.n) return;
    const int2 r = __ldg(g.rows + v);
    if (r.y - r.x > kWarpRow) list[atomicAdd(count, 1)] = make_int2(r.y - r.x, v);
}

// Smallest and largest edge label (for the label index: every label must lie
// in [0, kMaxIndexedLabels)).
__global__ void label_range_kernel(const int32_t *label, int64_t e, int *lo_hi) {
    int lo = INT_MAX, hi = INT_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < e; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = __ldg(label + i);
        lo = min(lo, x);
        hi = max(hi, x);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(kFull, lo, o));
        hi = max(hi, __shfl_xor_sync(kFull, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(lo_hi, lo);
        atomicMax(lo_hi + 1, hi);
    }
}

// MetaPath's label index, one warp per row (grid-stride): a stable counting
// sort of the row's neighbours by edge label.  Lane l keeps the counts and
// then the running output position of labels l and l + 32; each 32-entry
// chunk is scattered label by label with ballots, lanes of one label in lane
// order, so every label's block keeps row order.
__global__ void build_label_index_kernel(const DevGraph g, int32_t K, int32_t *off, int32_t *nbr) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < g.n; v += warps) {
        const int2 r = __ldg(g.rows + v);
        int32_t c0 = 0, c1 = 0;  // counts of labels lane and lane + 32
        for (int32_t base = r.x; base < r.y; base += 32) {
            const int32_t i = base + lane;
            const int32_t lab = i < r.y ? __ldg(g.label + i) : -1;
            for (int32_t l = 0; l < K; ++l) {
                const int32_t c = __popc(__ballot_sync(kFull, lab == l));
                if (l == lane) c0 += c;
                if (l == lane + 32) c1 += c;
            }
        }
        // exclusive scan over labels 0..K-1 held as (lane, c0) then (lane, c1)
        int32_t x0 = c0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(kFull, x0, o);
            if (lane >= o) x0 += y;
        }
        const int32_t total0 = __shfl_sync(kFull, x0, 31);
        int32_t x1 = c1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(kFull, x1, o);
            if (lane >= o) x1 += y;
        }
        int32_t b0 = x0 - c0, b1 = total0 + x1 - c1;  // block starts of labels lane, lane + 32
        int32_t *o = off + v * (int64_t)(K + 1);  // absolute positions in nbr: a walk step needs no row pair
        if (lane < K) o[lane] = r.x + b0;
        if (lane + 32 < K) o[lane + 32] = r.x + b1;
        if (lane == 0) o[K] = r.y;
        for (int32_t base = r.x; base < r.y; base += 32) {
            const int32_t i = base + lane;
            const int32_t lab = i < r.y ? __ldg(g.label + i) : -1;
            const int32_t nb = i < r.y ? __ldg(g.adj + i) : 0;
            for (int32_t l = 0; l < K; ++l) {
                const unsigned m = __ballot_sync(kFull, lab == l);
                if (!m) continue;
                const int32_t start = l < 32 ? __shfl_sync(kFull, b0, l) : __shfl_sync(kFull, b1, l - 32);
                if (lab == l) nbr[r.x + start + __popc(m & ((1u << lane) - 1u))] = nb;
                if (l == lane) b0 += __popc(m);
                if (l == lane + 32) b1 += __popc(m);
            }
        }
    }
}

// Sets *bad if an edge weight is negative or NaN, or a non-empty row has no
// positive weight (one warp per row, grid-stride).
__global__ void positive_rows_kernel(const DevGraph g, int *bad) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < g.n; v += warps) {
        const int2 r = __ldg(g.rows + v);
        bool neg = false, pos = false;
        for (int32_t i = r.x + lane; i < r.y; i += 32) {
            const double w = __ldg(g.weight + i);
            neg |= !(w >= 0.0);
            pos |= w > 0.0;
        }
        const bool any_neg = __any_sync(kFull, neg), any_pos = __any_sync(kFull, pos);
        if (lane == 0 && (any_neg || (r.y > r.x && !any_pos))) atomicOr(bad, 1);
    }
}

constexpr int kEdgeRun = 8;  // consecutive CSR entries per thread in the edge-set kernels

// Source vertex of CSR entry i: the largest v with rows[v].x <= i (rows of
// zero length share their start with the next row, so this is the row that
// holds i).
__device__ __forceinline__ int32_t row_of(const DevGraph &g, int64_t i) {
    int32_t lo = 0, hi = g.n - 1;
    while (lo < hi) {
        const int32_t mid = lo + ((hi - lo + 1) >> 1);
        if ((int64_t)__ldg(&g.rows[mid].x) <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Inserts every directed edge (v, adj[i]) into the set.  Each thread takes
// kEdgeRun consecutive entries: one search for the first entry's row, then
// it walks forward row by row.
__global__ void build_edge_set_kernel(DevGraph g, unsigned long long *set, int32_t bits) {
    const uint32_t mask = (1u << bits) - 1u;
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kEdgeRun;
    if (first >= g.e) return;
    int32_t v = row_of(g, first);
    int2 r = __ldg(g.rows + v);
    const int64_t last = min(first + kEdgeRun, g.e);
    for (int64_t i = first; i < last; ++i) {
        while (i >= r.y) r = __ldg(g.rows + ++v);
        const unsigned long long k = edge_key(v, __ldg(g.adj + i));
        uint32_t h = edge_slot(k, bits);
        for (uint32_t probe = 0; probe <= mask; ++probe) {
            const unsigned long long old = atomicCAS(set + h, kEdgeEmpty, k);
            if (old == kEdgeEmpty || old == k) break;
            h = (h + 1) & mask;
        }
    }
}

// DevGraph::lab_fat: one warp per row, label block by label block; the
// next label of block l is next.label[l] (-1: not in the schema, or no edge
// carries it).
__global__ void build_lab_fat_kernel(const DevGraph g, const LabelNext next, int4 *fat) {
    const int lane = threadIdx.x & 31;
    const int K = g.lab_k;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < g.n; v += warps) {
        const int32_t *o = g.lab_off + v * (int64_t)(K + 1);
        for (int32_t l = 0; l < K; ++l) {
            const int32_t w = next.label[l];
            const int32_t b = __ldg(o + l), end = __ldg(o + l + 1);
            for (int32_t i = b + lane; i < end; i += 32) {
                const int32_t u = __ldg(g.lab_nbr + i);
                int32_t x = 0, y = 0;
                if (w >= 0) {
                    const int32_t *ou = g.lab_off + (int64_t)u * (K + 1) + w;
                    x = __ldg(ou);
                    y = __ldg(ou + 1);
                }
                fat[i] = make_int4(u, x, y, 0);
            }
        }
    }
}

// The uniform moves' adjacency with the neighbours' row pairs (DevGraph::fat).
__global__ void build_fat_kernel(DevGraph g, int4 *fat) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.e) return;
    const int32_t v = __ldg(g.adj + i);
    const int2 r = __ldg(g.rows + v);
    fat[i] = make_int4(v, r.x, r.y, 0);
}

// Clears *symmetric if some edge's reverse is missing.
__global__ void edge_symmetry_kernel(DevGraph g, int *symmetric) {
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kEdgeRun;
    if (first >= g.e) return;
    int32_t v = row_of(g, first);
    int2 r = __ldg(g.rows + v);
    const int64_t last = min(first + kEdgeRun, g.e);
    for (int64_t i = first; i < last; ++i) {
        while (i >= r.y) r = __ldg(g.rows + ++v);
        if (!edge_exists(g, __ldg(g.adj + i), v)) {
            atomicAnd(symmetric, 0);
            return;
        }
    }
}

}  // namespace

cudaError_t launch_collect_long_rows(const DevGraph &g, int2 *list, int *count, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    collect_long_rows_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, list, count);
    return cudaGetLastError();
}

cudaError_t launch_build_alias(const DevGraph &g, int unit, AliasSlot *out, const int32_t *long_rows,
                               int32_t n_long, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_alias_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    if (n_long > 0) build_alias_warp_kernel<<<(unsigned)n_long, 32, 0, st>>>(g, unit, out, long_rows);
    return cudaGetLastError();
}

cudaError_t launch_build_prefix(const DevGraph &g, int unit, double *out, const int32_t *long_rows,
                                int32_t n_long, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_prefix_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    if (n_long > 0) build_prefix_warp_kernel<<<(unsigned)n_long, 32, 0, st>>>(g, unit, out, long_rows);
    return cudaGetLastError();
}

cudaError_t launch_build_max(const DevGraph &g, int unit, double *out, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    build_max_kernel<<<blocks_for(g.n), 256, 0, st>>>(g, unit, out);
    return cudaGetLastError();
}

cudaError_t launch_positive_rows(const DevGraph &g, int *bad, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>(((int64_t)g.n * 32 + 255) / 256, 152 * 64);
    positive_rows_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, bad);
    return cudaGetLastError();
}

cudaError_t launch_label_range(const int32_t *label, int64_t e, int *lo_hi, cudaStream_t st) {
    if (e <= 0) return cudaSuccess;
    label_range_kernel<<<1024, 256, 0, st>>>(label, e, lo_hi);
    return cudaGetLastError();
}

cudaError_t launch_build_label_index(const DevGraph &g, int32_t K, int32_t *off, int32_t *nbr, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>(((int64_t)g.n * 32 + 255) / 256, 152 * 64);
    build_label_index_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, K, off, nbr);
    return cudaGetLastError();
}

cudaError_t launch_build_edge_set(const DevGraph &g, unsigned long long *set, int32_t bits, int *symmetric,
                                  cudaStream_t st) {
    if (g.e <= 0) return cudaSuccess;
    const unsigned grid = blocks_for((g.e + kEdgeRun - 1) / kEdgeRun);
    build_edge_set_kernel<<<grid, 256, 0, st>>>(g, set, bits);
    DevGraph gs = g;
    gs.edges = set;
    gs.edge_bits = bits;
    edge_symmetry_kernel<<<grid, 256, 0, st>>>(gs, symmetric);
    return cudaGetLastError();
}

cudaError_t launch_build_lab_fat(const DevGraph &g, const LabelNext &next, int4 *fat, cudaStream_t st) {
    if (g.n <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>(((int64_t)g.n * 32 + 255) / 256, 152 * 64);
    build_lab_fat_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, next, fat);
    return cudaGetLastError();
}

cudaError_t launch_build_fat(const DevGraph &g, int4 *fat, cudaStream_t st) {
    if (g.e <= 0) return cudaSuccess;
    build_fat_kernel<<<blocks_for(g.e), 256, 0, st>>>(g, fat);
    return cudaGetLastError();
}

cudaError_t launch_validate_graph(const int64_t *row, const int32_t *adj, int32_t n, int64_t e, int check_sorted,
                                  int2 *rows_out, int *bad, int *max_degree, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    validate_kernel<<<blocks_for((int64_t)n * 32), 256, 0, st>>>(row, adj, n, e, check_sorted, rows_out, bad, max_degree);
    return cudaGetLastError();
}

}  // namespace trw
