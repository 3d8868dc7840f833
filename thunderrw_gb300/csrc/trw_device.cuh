// trw_device.cuh -- device-side building blocks shared by the walk and
// table-builder kernels: Philox4x32-10, SFMT's u32->double conversions, the
// HBM graph view, the app hooks and the launch parameters.
//
// All translation units including this header are compiled with
// --fmad=false: every double operation is one IEEE round-to-nearest op, the
// same arithmetic as the reference's x86-64 build.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace trw {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11).  key = seed; counter = (block, step,
// walker lo, walker hi).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

constexpr uint32_t kTermBlock = 0x80000000u;

__device__ __forceinline__ uint4 draw_block(uint64_t seed, uint64_t walker, uint32_t step, uint32_t block) {
    return philox4x32_10(make_uint4(block, step, (uint32_t)walker, (uint32_t)(walker >> 32)),
                         (uint32_t)seed, (uint32_t)(seed >> 32));
}

__device__ __forceinline__ uint32_t word(const uint4 &v, uint32_t i) {
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Sequential draws of one (walker, step) move: draw d is word d%4 of block d/4.
struct DrawCursor {
    uint64_t seed, walker;
    uint32_t step, draw;
    uint4 buf;
    __device__ __forceinline__ DrawCursor(uint64_t s, uint64_t w, uint32_t st, const uint4 &first)
        : seed(s), walker(w), step(st), draw(0), buf(first) {}
    __device__ __forceinline__ uint32_t next() {
        if (draw && (draw & 3) == 0) buf = draw_block(seed, walker, step, draw >> 2);
        return word(buf, draw++ & 3);
    }
};

// SFMT.h:193-228: real1 = v / (2^32 - 1) via the rounded reciprocal, real2 = v * 2^-32.
__device__ __forceinline__ double real1(uint32_t v) { return (double)v * (1.0 / 4294967295.0); }
__device__ __forceinline__ double real2(uint32_t v) { return (double)v * (1.0 / 4294967296.0); }

// real2(u) <= x without the FP64 pipe (GB300 issues one warp-wide FP64
// instruction per 64 cycles per SM sub-partition).  real2(u) = u * 2^-32
// exactly, so the test is u <= floor(x * 2^32), read off x's IEEE fields.
__device__ __forceinline__ bool real2_le(uint32_t u, double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
    if (b >> 63) return u == 0 && (b << 1) == 0;  // x < 0: never; x = -0.0: u = 0 only
    if (e == 0x7FFu) return frac == 0;            // +inf: always; NaN: never
    if (e >= 1023u) return true;                  // x >= 1 > real2(u)
    const unsigned long long m = e ? (frac | (1ull << 52)) : frac;
    const uint32_t shift = 1043u - (e ? e : 1u);  // x * 2^32 = m * 2^-shift
    return (unsigned long long)u <= (shift >= 64u ? 0ull : m >> shift);
}

// ---------------------------------------------------------------------------
// Graph view in HBM.
//   rows[v]  = (row_ptr[v], row_ptr[v+1]) as one 8-byte pair: a single aligned
//              load per step (the offset_pair_ of graph.cpp:86-91 at half size)
//   adj      = neighbour ids, sorted per row
//   alias    = 16-byte AliasSlot rows, one aligned 16-byte load per draw
// ---------------------------------------------------------------------------
struct AliasSlot {
    double prob;
    int32_t first;
    int32_t second;
};
static_assert(sizeof(AliasSlot) == 16, "AliasSlot must be 16 bytes");

struct DevGraph {
    const int2 *rows;
    const int32_t *adj;
    const double *weight;
    const int32_t *label;
    const AliasSlot *alias;
    const double *prefix;
    const double *rmax;
    // Node2Vec's neighbour test: an open-addressing set of the directed edges
    // (u, v) as (u << 32 | v), 2^edge_bits slots, kEdgeEmpty = free; null
    // until the first Node2Vec walk builds it.  edge_symmetric: every edge's
    // reverse is present.
    const unsigned long long *edges;
    int32_t edge_bits;
    int32_t edge_symmetric;
    // MetaPath's label index (built by the first MetaPath ITS walk when every
    // label lies in [0, lab_k), lab_k <= 64; null otherwise): lab_nbr holds
    // each row's neighbours stably sorted by edge label (row order inside a
    // label), lab_off[v * (lab_k + 1) + l] the position in lab_nbr where label
    // l's block of row v starts and lab_off[v * (lab_k + 1) + lab_k] the row's
    // end (lab_nbr is laid out like adj, so these are CSR positions).
    const int32_t *lab_nbr;
    const int32_t *lab_off;
    int32_t lab_k;
    // The label index with the next step's positions folded in, for a walk
    // whose schema names each label at most once (so the label an entry's
    // edge carries fixes the label its vertex's next step wants): entry j =
    // {lab_nbr[j], lab_off[v * (lab_k + 1) + w], lab_off[... + w + 1], 0}
    // with v = lab_nbr[j] and w the label after j's in the schema ({v, 0, 0}
    // if w has no edges); one 16-byte load gives a step its vertex and the
    // next step's block (null unless built for this walk's schema).
    const int4 *lab_fat;
    // the adjacency is at least twice the L2: uniform moves read it evict-first
    int32_t adj_streams;
    // The adjacency with the row pairs folded in, for uniform and max-weight
    // rejection moves on graphs whose row pairs do not stay in L2: entry i
    // holds {adj[i], rows[adj[i]].x, rows[adj[i]].y, 0}, so one 16-byte load
    // gives the next vertex and the row it will sample from (null if not
    // built).
    const int4 *fat;
    int32_t n;
    int64_t e;
};

constexpr unsigned long long kEdgeEmpty = ~0ull;  // (0xffffffff, 0xffffffff) is no edge: ids < 2^31

__device__ __forceinline__ unsigned long long edge_key(int32_t u, int32_t v) {
    return ((unsigned long long)(uint32_t)u << 32) | (uint32_t)v;
}

__device__ __forceinline__ uint32_t edge_slot(unsigned long long k, int32_t bits) {
    return (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> (64 - bits));
}

// Whether the directed edge (u, v) exists (u's list holds v).  The set is at
// most two-thirds full, so a free slot ends every probe sequence.
// L2 eviction priority (createpolicy + ld .L2::cache_hint, PTX ISA 7.4 for
// sm_80 and later).  On a graph whose adjacency is several times the L2, a
// uniform step's random adjacency read brings in a fresh line (about
// 2.4 TB/s of them in the sparse PPR walk) that is rarely read again before
// it leaves L2; marked evict-first it stops pushing out the lines that are
// read again: the in-flight queries' visit tables (whose key loads are
// marked evict-last) and the hot rows.  Measured on GB300: the sparse PPR
// walk on R-MAT 2^22 (0.5 GB of adjacency) 5.55 -> 5.14 ms.  Where the data
// is re-read from L2 the same hint costs: DeepWalk on Chung-Lu 2^18 (graph
// and alias table in L2) 0.27 -> 0.41 ms with its alias reads marked,
// Node2Vec 22.5 -> 23.3 ms with its candidate and edge-set reads marked; so
// only the uniform move's adjacency read takes it, and only on such graphs.
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// read-only data read once (the non-coherent path, evict-first in L2)
__device__ __forceinline__ int32_t ld_once(const int32_t *a) {
    int32_t v;
    asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(l2_evict_first()));
    return v;
}
__device__ __forceinline__ int4 ld_once(const int4 *a) {
    int4 v;
    asm volatile("ld.global.nc.L2::cache_hint.v4.b32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(a), "l"(l2_evict_first()));
    return v;
}
// data written by atomics during the kernel, read through L2 and kept there
__device__ __forceinline__ int32_t ldcg_keep(const int32_t *a) {
    int32_t v;
    asm volatile("ld.global.cg.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(l2_evict_last()));
    return v;
}

__device__ __forceinline__ bool edge_exists(const DevGraph &g, int32_t u, int32_t v) {
    const unsigned long long k = edge_key(u, v);
    const uint32_t mask = (1u << g.edge_bits) - 1u;
    uint32_t h = edge_slot(k, g.edge_bits);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long x = __ldg(g.edges + h);
        if (x == k) return true;
        if (x == kEdgeEmpty) return false;
        h = (h + 1) & mask;
    }
    return false;
}

// kLabelIndex: MetaPath's dynamic ITS answered from the label index (an
// engine-internal sampler; it shares the ITS launch-shape slot)
enum Sampler : int { kUniform = 0, kITS = 1, kAlias = 2, kRejection = 3, kMaxRejection = 4, kLabelIndex = 5 };
constexpr int kMaxIndexedLabels = 64;
enum Update : int { kFixedLength = 0, kGeometric = 1 };
enum WeightKind : int { kEdgeWeight = 0, kUnitWeight = 1, kNode2Vec = 2, kLabelSchema = 3 };

constexpr int kMaxSchema = 64;
constexpr uint32_t kMaxTrials = 1u << 20;

enum DeviceError : int { kErrTrials = 1, kErrVertex = 2, kErrCapacity = 4 };

struct WalkParams {
    DevGraph g;
    // app
    int32_t length;       // l_
    int32_t schema_len;
    double p_w, q_w, n2v_max, tp, max_weight;
    uint32_t tp_max;  // largest draw v with real1(v) <= tp (real1 is monotonic in v)
    // max-weight rejection with walker-independent weight values (Node2Vec's
    // n2v_max, 1/p, 1, 1/q; PPR's 1): accept <=> draw u <= accept_max[k] with
    // k the weight's class, the largest u with real2(u) * max_weight <= w_k
    uint32_t accept_max[4];
    uint64_t seed;
    int32_t static_unit;  // static rejection with unit weights (PPR)
    int32_t schema[kMaxSchema];
    // walkers
    const int32_t *sources;
    int64_t num_walkers;
    int64_t per_query;    // > 0: walker i starts at sources[i / per_query]
    int64_t id_base;
    // outputs
    int32_t *paths;
    int32_t path_cap;
    int32_t path_vec;     // paths 16-byte aligned and path_cap % 4 == 0: the thread kernels store 4 entries at a time
    int32_t *lengths;
    int32_t *counts;
    // engine state
    unsigned long long *queue_head;
    unsigned long long *steps;
    int *error;
    // dynamic alias scratch: one table of max_degree slots per warp
    AliasSlot *alias_scratch;
    int64_t alias_scratch_stride;
    // sparse visit counts: per query an open-addressing table of 2^table_bits
    // slots stored as 2^table_bits keys (vertex + 1, 0 = empty) followed by
    // 2^table_bits counts (visits minus one).  Keys and counts live in
    // separate sectors so that reading a hot key never queues behind the
    // atomic adds to its count.
    int32_t *table;
    int32_t table_bits;
};

// Adds `inc` visits of vertex v to a query's table t (keys t[0..C), counts
// t[C..2C)): linear probing on key v + 1, 0 = empty.  A slot's count holds
// its visits minus one: the CAS that claims the slot stands for the first.
// Which slots end up occupied does not depend on the insertion order; only
// the order of keys inside a run of occupied slots does.
__device__ __forceinline__ void table_add(int32_t *t, int32_t bits, int32_t v, int inc, int *error) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t h = ((uint32_t)v * 0x9E3779B1u) >> (32 - bits);
    const int32_t key = v + 1;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        int k = __ldcg(t + h);
        if (k == 0) {
            k = atomicCAS(t + h, 0, key);
            if (k == 0) {  // claimed
                if (inc > 1) atomicAdd(t + mask + 1 + h, inc - 1);
                return;
            }
        }
        if (k == key) { atomicAdd(t + mask + 1 + h, inc); return; }
        h = (h + 1) & mask;
    }
    atomicOr(error, kErrCapacity);  // table full: every slot holds another vertex
}

// Records a move to `v` for walker query q (dense counts or the sparse
// table).  Lanes of the warp that record the same (query, vertex) at the same
// time are merged first (walkers of one query leave the same vertices
// together), so each distinct pair costs one memory update per warp.
__device__ __forceinline__ void record_visit(const WalkParams &p, int64_t q, int32_t v) {
    if (!p.table && !p.counts) return;
    const unsigned active = __activemask();
    const unsigned long long key = ((unsigned long long)q << 32) | (uint32_t)v;
    const unsigned peers = __match_any_sync(active, key);
    if ((threadIdx.x & 31) != __ffs(peers) - 1) return;
    const int inc = __popc(peers);
    if (p.table)
        table_add(p.table + (q << (p.table_bits + 1)), p.table_bits, v, inc, p.error);
    else atomicAdd(p.counts + q * (int64_t)p.g.n + v, inc);
}

// Graph::is_neighbor (graph.h:180-199): binary search for the higher-degree
// endpoint in the lower-degree endpoint's sorted list (ties search u in v's).
__device__ __forceinline__ bool is_neighbor(const DevGraph &g, int32_t u, int2 ru, int32_t v, int2 rv) {
    int32_t du = ru.y - ru.x, dv = rv.y - rv.x;
    if (du < dv) { int32_t t = u; u = v; v = t; int2 tr = ru; ru = rv; rv = tr; }
    const int32_t *nb = g.adj + rv.x;
    int32_t lo = 0, hi = rv.y - rv.x - 1;
    while (lo <= hi) {
        const int32_t mid = lo + ((hi - lo) >> 1);
        const int32_t x = __ldg(nb + mid);
        if (x == u) return true;
        if (x > u) hi = mid - 1; else lo = mid + 1;
    }
    return false;
}

// is_neighbor(prev, nbr) as Node2Vec's hook calls it (node2vec.cpp:186-193).
// With the edge set: on a symmetric graph the answer is edge (prev, nbr); on
// others the reference's choice of list (the lower-degree endpoint's,
// graph.h:181-183) needs both degrees, then one lookup.  Without it: the
// binary search.
__device__ __forceinline__ bool n2v_neighbor(const DevGraph &g, int32_t prev, int2 prev_row, int32_t nbr) {
    if (g.edges) {
        if (g.edge_symmetric) return edge_exists(g, prev, nbr);
        const int2 rn = __ldg(g.rows + nbr);
        // is_neighbor(u = prev, v = nbr): swap if deg(u) < deg(v), then look for u in v's list
        const bool swap = (prev_row.y - prev_row.x) < (rn.y - rn.x);
        return swap ? edge_exists(g, prev, nbr) : edge_exists(g, nbr, prev);
    }
    const int2 rn = __ldg(g.rows + nbr);
    return is_neighbor(g, prev, prev_row, nbr, rn);
}

// The weight hook of the app (node2vec.cpp:182-196, metapath.cpp:22-30,
// deepwalk.cpp:19-21, ppr.cpp:95-97) for the edge (cur -> nbr) at eid.
// `len` and `prev` are the walker's length_ and seq_[length_-2].
template <int WK>
__device__ __forceinline__ double app_weight(const WalkParams &p, int32_t len, int32_t prev, int2 prev_row,
                                             int32_t nbr, int64_t eid) {
    if (WK == kEdgeWeight) return __ldg(p.g.weight + eid);
    if (WK == kUnitWeight) return 1.0;
    if (WK == kLabelSchema) return __ldg(p.g.label + eid) != p.schema[(len - 1) % p.schema_len] ? 0.0 : 1.0;
    // Node2Vec
    if (len == 1) return p.n2v_max;
    if (nbr == prev) return p.p_w;
    return n2v_neighbor(p.g, prev, prev_row, nbr) ? 1.0 : p.q_w;
}

// Node2Vec's weight as a class index into accept_max: 0 n2v_max (first move),
// 1 return (1/p), 2 common neighbour (1), 3 otherwise (1/q); the same cases
// as app_weight<kNode2Vec>.
__device__ __forceinline__ int n2v_class(const WalkParams &p, int32_t len, int32_t prev, int2 prev_row,
                                         int32_t nbr) {
    if (len == 1) return 0;
    if (nbr == prev) return 1;
    return n2v_neighbor(p.g, prev, prev_row, nbr) ? 2 : 3;
}

// Node2Vec's max-weight rejection test for acceptance draw u: u <=
// accept_max[class of nbr].  When the candidate is neither the first move
// nor a return, its class is 2 or 3 and the neighbour test (a probe of the
// edge set) only matters for draws between the two classes' thresholds:
// below both the move is accepted and above both rejected, whichever class
// it is.  The decision is the one the hook's weight gives
// (rejection_sampling.h:384-389, node2vec.cpp:182-196) with the probe skipped
// where it cannot change it.
__device__ __forceinline__ bool n2v_accept(const WalkParams &p, int32_t len, int32_t prev, int2 prev_row,
                                           int32_t nbr, uint32_t u) {
    if (len == 1) return u <= p.accept_max[0];
    if (nbr == prev) return u <= p.accept_max[1];
    const uint32_t lo = min(p.accept_max[2], p.accept_max[3]), hi = max(p.accept_max[2], p.accept_max[3]);
    if (u <= lo) return true;
    if (u > hi) return false;
    return u <= p.accept_max[n2v_neighbor(p.g, prev, prev_row, nbr) ? 2 : 3];
}

// The update hook: length_ == l_, or PPR's real1(termination draw) <= tp.
template <int U>
__device__ __forceinline__ bool app_update(const WalkParams &p, uint64_t wid, int32_t len) {
    if (U == kFixedLength) return len == p.length;
    const uint4 t = draw_block(p.seed, wid, (uint32_t)len, kTermBlock);
    return t.x <= p.tp_max;  // == (real1(t.x) <= p.tp), without the FP64 pipe
}

// Utility::upper_bound_branchless (utility.h:18-27): number of entries <= t.
__device__ __forceinline__ int32_t upper_bound_bl(const double *src, int32_t n, double t) {
    const double *base = src;
    while (n > 1) {
        const int32_t half = n >> 1;
        base = (__ldg(base + half) <= t) ? base + half : base;
        n -= half;
    }
    return (int32_t)((__ldg(base) <= t) + (base - src));
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace trw
