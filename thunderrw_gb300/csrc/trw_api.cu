// trw_api.cu -- the extern "C" boundary of libtrw_gpu.so (include/trw.h).
//
// Owns the graph's HBM arrays, the static tables and the per-call engine
// state, maps the reference's (app, mode, sampler) triple (types.h:41-59,
// creeper.h:700-788) onto the two kernel families, and stages host buffers.
#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "trw.h"
#include "trw_batch.h"
#include "trw_device.cuh"
#include "trw_internal.h"

using namespace trw;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define TRW_CUDA(call)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(TRW_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

bool is_device_ptr(const void *ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device allocation that frees itself.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t ensure(size_t want) {
        if (bytes >= want) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
};

// One in-flight call's device state; reused once its event has completed.
struct EngineSlot {
    unsigned long long *queue_head = nullptr;  // points into the graph's state block
    unsigned long long *steps = nullptr;
    cudaEvent_t done = nullptr;
    bool used = false;
};

constexpr int kEngineSlots = 64;
constexpr int kMaxRanges = 16;  // walker ranges of a host-output walk (the pipelines' event arrays)
// Query ranges of a sparse PPR batch with host outputs.  The 4096 x 10^4
// batch on R-MAT 2^22 takes 9.8 / 9.17 / 9.24 ms end to end at 4 / 8 / 16
// equal ranges (each range boundary costs a walk tail; too few leave the
// last range's copy exposed) and 8.80 ms as 10 ranges weighted
// 1,1,2,2,2,2,2,2,1,1: the small first ranges start the copies early and
// the small last ones leave little copy after the final walk.  Batches with
// fewer than 16 units of 8 walkers per lane use at most kPprRanges equal
// ranges.
constexpr int kPprRanges = 8;
// Post-processing chunks of a host-output batch: 2^14 slots a CTA (2^16 for
// device outputs, where the whole batch fills the GPU with tables).
constexpr int32_t kPprRangeChunkBits = 14;
constexpr int kPprSplit[] = {1, 1, 2, 2, 2, 2, 2, 2, 1, 1};
constexpr int kPprSplitUnits = 16;  // sum of kPprSplit

int app_weight_kind(int app) {
    switch (app) {
    case TRW_APP_PPR: return kUnitWeight;
    case TRW_APP_NODE2VEC: return kNode2Vec;
    case TRW_APP_METAPATH: return kLabelSchema;
    default: return kEdgeWeight;
    }
}

}  // namespace

struct trw_graph {
    int device = 0;
    int num_sms = 1;
    int32_t n = 0;
    int64_t e = 0;
    int32_t max_degree = 0;
    bool sorted = false;
    int2 *rows = nullptr;
    int32_t *adj = nullptr;
    double *weight = nullptr;
    int32_t *label = nullptr;
    AliasSlot *alias = nullptr;
    double *prefix = nullptr;
    double *rmax = nullptr;
    int alias_kind = -1, prefix_kind = -1, rmax_kind = -1;
    // Node2Vec's edge set (built by its first walk); edge_state 0 = not yet,
    // 1 = built, -1 = no room for it (the walks then binary-search the lists)
    unsigned long long *edges = nullptr;
    int32_t edge_bits = 0;
    // rows longer than 32 entries, longest first (the warp table builders'
    // work list); n_long < 0 until first needed
    int32_t *long_rows = nullptr;
    int32_t n_long = -1;
    // MetaPath's label index (built by its first dynamic-ITS walk); lab_state
    // 0 = not yet, 1 = built, -1 = labels outside [0, 64) or no room
    int32_t *lab_nbr = nullptr;
    int32_t *lab_off = nullptr;
    int32_t lab_k = 0;
    int lab_state = 0;
    // every edge weight >= 0 and every non-empty row with a positive one:
    // 0 = not checked yet, 1 = yes, -1 = no
    int positive_rows = 0;
    int32_t edge_symmetric = 0;
    int edge_state = 0;
    // the adjacency with row pairs (DevGraph::fat), built by the first
    // uniform or max-weight rejection thread-engine walk on a graph whose row
    // pairs outgrow half the L2; fat_state 0 = not yet, 1 = built, -1 = not
    // built (the walks then read the row pairs)
    int4 *fat = nullptr;
    int fat_state = 0;
    int32_t adj_streams = 0;  // DevGraph::adj_streams (set at creation)
    // the label index with the next step's positions (DevGraph::lab_fat),
    // built by trw_walk for the schema in lab_fat_schema; lab_fat_state 0 =
    // never decided, 1 = built (for that schema), -1 = not built
    int4 *lab_fat = nullptr;
    int lab_fat_state = 0;
    std::vector<int32_t> lab_fat_schema;
    // engine state block: [kEngineSlots x (queue, steps)] + error word
    unsigned long long *state = nullptr;
    int *error = nullptr;
    EngineSlot slots[kEngineSlots];
    int next_slot = 0;
    DevBuf stage;
    DevBuf alias_scratch;
    cudaEvent_t scratch_done = nullptr;
    LaunchShape shape[5];
    // sparse PPR: per-query visit tables (kept all-zero between batches),
    // per-query distinct-vertex counts and output staging
    DevBuf ppr_tables;
    int32_t ppr_bits = 0;
    int64_t ppr_queries = 0;
    bool ppr_dirty = false;  // a batch stopped between its walk and its emit
    cudaEvent_t ppr_done = nullptr;  // last sparse batch's emit: the tables are free after it
    cudaEvent_t tables_done = nullptr;  // last static-table build: walks on any stream wait for it
    // optional per-call timing: events around the walk launch and after the
    // post-processing launches of the last call
    bool profile = false;
    cudaEvent_t ev_walk0 = nullptr, ev_walk1 = nullptr, ev_post1 = nullptr;
    bool have_post = false;
    DevBuf ppr_distinct;
    DevBuf stage_out;
    // sparse PPR into host buffers: a second compute stream and a copy
    // stream, per-range events (offsets scanned, range finished) and pinned
    // words receiving each range's last offset
    cudaStream_t aux_stream = nullptr, copy_stream = nullptr;
    cudaEvent_t range_done[kMaxRanges] = {}, offsets_done[kMaxRanges] = {};
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int64_t *h_ends = nullptr;
    std::mutex mu;
};

namespace {

void destroy_graph(trw_graph *g) {
    if (!g) return;
    cudaFree(g->rows); cudaFree(g->adj); cudaFree(g->weight); cudaFree(g->label);
    cudaFree(g->alias); cudaFree(g->prefix); cudaFree(g->rmax); cudaFree(g->state); cudaFree(g->edges);
    cudaFree(g->long_rows); cudaFree(g->lab_nbr); cudaFree(g->lab_off); cudaFree(g->fat); cudaFree(g->lab_fat);
    for (auto &s : g->slots) if (s.done) cudaEventDestroy(s.done);
    if (g->scratch_done) cudaEventDestroy(g->scratch_done);
    for (cudaEvent_t e : {g->ev_walk0, g->ev_walk1, g->ev_post1, g->ppr_done, g->tables_done})
        if (e) cudaEventDestroy(e);
    for (int r = 0; r < kMaxRanges; ++r) {
        if (g->range_done[r]) cudaEventDestroy(g->range_done[r]);
        if (g->offsets_done[r]) cudaEventDestroy(g->offsets_done[r]);
    }
    if (g->ev_fork) cudaEventDestroy(g->ev_fork);
    if (g->ev_join) cudaEventDestroy(g->ev_join);
    if (g->aux_stream) cudaStreamDestroy(g->aux_stream);
    if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
    if (g->h_ends) cudaFreeHost(g->h_ends);
    delete g;
}

DevGraph dev_view(const trw_graph *g) {
    DevGraph d;
    d.rows = g->rows; d.adj = g->adj; d.weight = g->weight; d.label = g->label;
    d.alias = g->alias; d.prefix = g->prefix; d.rmax = g->rmax; d.n = g->n; d.e = g->e;
    d.edges = g->edge_state == 1 ? g->edges : nullptr;
    d.edge_bits = g->edge_bits;
    d.edge_symmetric = g->edge_symmetric;
    d.lab_nbr = g->lab_state == 1 ? g->lab_nbr : nullptr;
    d.lab_off = g->lab_state == 1 ? g->lab_off : nullptr;
    d.lab_k = g->lab_state == 1 ? g->lab_k : 0;
    d.fat = g->fat_state == 1 ? g->fat : nullptr;
    d.lab_fat = nullptr;  // per walk: lab_fat_for()
    d.adj_streams = g->adj_streams;
    return d;
}

// MetaPath's label index: each row's neighbours stably sorted by label, plus
// per-row label offsets, so dynamic ITS over the label filter reads one entry
// instead of scanning the row.  Only for labels in [0, 64); otherwise, or if
// the device has no room, the walks keep scanning label rows.
int build_label_index(trw_graph *g, cudaStream_t st) {
    if (g->lab_state != 0 || g->e <= 0 || !g->label) return TRW_OK;
    int *d_lh = nullptr;
    TRW_CUDA(cudaMalloc(&d_lh, 2 * sizeof(int)));
    const int init[2] = {INT_MAX, INT_MIN};
    TRW_CUDA(cudaMemcpyAsync(d_lh, init, sizeof init, cudaMemcpyHostToDevice, st));
    TRW_CUDA(launch_label_range(g->label, g->e, d_lh, st));
    int lh[2] = {0, 0};
    TRW_CUDA(cudaMemcpyAsync(lh, d_lh, sizeof lh, cudaMemcpyDeviceToHost, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    cudaFree(d_lh);
    if (lh[0] < 0 || lh[1] >= kMaxIndexedLabels) { g->lab_state = -1; return TRW_OK; }
    const int32_t K = lh[1] + 1;
    const size_t b_off = sizeof(int32_t) * (size_t)g->n * (size_t)(K + 1);
    const size_t b_nbr = sizeof(int32_t) * (size_t)g->e;
    size_t free_b = 0, total_b = 0;
    TRW_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (b_off + b_nbr + (size_t(1) << 30) > free_b || cudaMalloc(&g->lab_off, b_off) != cudaSuccess ||
        cudaMalloc(&g->lab_nbr, b_nbr) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(g->lab_off);
        cudaFree(g->lab_nbr);
        g->lab_off = g->lab_nbr = nullptr;
        g->lab_state = -1;
        return TRW_OK;
    }
    TRW_CUDA(launch_build_label_index(dev_view(g), K, g->lab_off, g->lab_nbr, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    g->lab_k = K;
    g->lab_state = 1;
    return TRW_OK;
}

// The adjacency with the neighbours' row pairs folded in (16 bytes per
// edge): a move reads one entry instead of the row pair and then the entry.
// Worth its memory only where the row pairs are DRAM reads: when they take
// more than half the L2 (R-MAT 2^24: 128 MB of row pairs, Node2Vec's DRAM
// traffic per step falls; R-MAT 2^22: 32 MB, L2 hits, no change measured).
// If the device has no room for it the walks keep the two loads.
int build_fat_adjacency(trw_graph *g, cudaStream_t st) {
    if (g->fat_state != 0 || g->e <= 0) return TRW_OK;
    // TRW_FAT_ADJACENCY=0 / 1 turns the rule off / on for every graph
    const char *force = getenv("TRW_FAT_ADJACENCY");
    int l2 = 0;
    TRW_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, g->device));
    const bool want = force && *force ? *force == '1' : sizeof(int2) * (size_t)g->n > (size_t)l2 / 2;
    if (!want) { g->fat_state = -1; return TRW_OK; }
    const size_t bytes = sizeof(int4) * (size_t)g->e;
    size_t free_b = 0, total_b = 0;
    TRW_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bytes + (size_t(1) << 30) > free_b || cudaMalloc(&g->fat, bytes) != cudaSuccess) {
        cudaGetLastError();
        g->fat = nullptr;
        g->fat_state = -1;
        return TRW_OK;
    }
    TRW_CUDA(launch_build_fat(dev_view(g), g->fat, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    g->fat_state = 1;
    return TRW_OK;
}

// Node2Vec's neighbour test as one hash probe instead of a binary search:
// the set of directed edges, at most two-thirds full (2^bits >= 1.5 e).  If
// the device has no room for it the walks keep the binary search.
int build_edge_set(trw_graph *g, cudaStream_t st) {
    if (g->edge_state != 0 || g->e <= 0) return TRW_OK;
    int32_t bits = 10;
    while (bits < 32 && (double)(1ull << bits) < 1.5 * (double)g->e) ++bits;
    if (bits > 31) { g->edge_state = -1; return TRW_OK; }
    const size_t bytes = sizeof(unsigned long long) << bits;
    size_t free_b = 0, total_b = 0;
    TRW_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bytes + (size_t(1) << 30) > free_b || cudaMalloc(&g->edges, bytes) != cudaSuccess) {
        cudaGetLastError();
        g->edges = nullptr;
        g->edge_state = -1;
        return TRW_OK;
    }
    int *d_sym = nullptr;
    TRW_CUDA(cudaMalloc(&d_sym, sizeof(int)));
    const int one = 1;
    TRW_CUDA(cudaMemcpyAsync(d_sym, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    TRW_CUDA(cudaMemsetAsync(g->edges, 0xFF, bytes, st));
    TRW_CUDA(launch_build_edge_set(dev_view(g), g->edges, bits, d_sym, st));
    int sym = 0;
    TRW_CUDA(cudaMemcpyAsync(&sym, d_sym, sizeof(int), cudaMemcpyDeviceToHost, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    cudaFree(d_sym);
    g->edge_bits = bits;
    g->edge_symmetric = sym;
    g->edge_state = 1;
    return TRW_OK;
}

// The rows the warp builders take (longer than 32 entries), longest first:
// each gets a warp of its own block, so the hub rows -- whose alias pairing
// and prefix chains are sequential double arithmetic -- start first and
// run on different SMs instead of sharing one CTA.
int collect_long_rows(trw_graph *g, cudaStream_t st) {
    int2 *d_list = nullptr;
    int *d_count = nullptr;
    TRW_CUDA(cudaMalloc(&d_list, sizeof(int2) * (size_t)g->n));
    TRW_CUDA(cudaMalloc(&d_count, sizeof(int)));
    TRW_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
    TRW_CUDA(launch_collect_long_rows(dev_view(g), d_list, d_count, st));
    int count = 0;
    TRW_CUDA(cudaMemcpyAsync(&count, d_count, sizeof(int), cudaMemcpyDeviceToHost, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    std::vector<int2> list((size_t)count);
    if (count) TRW_CUDA(cudaMemcpy(list.data(), d_list, sizeof(int2) * (size_t)count, cudaMemcpyDeviceToHost));
    cudaFree(d_list);
    cudaFree(d_count);
    std::sort(list.begin(), list.end(), [](const int2 &a, const int2 &b) { return a.x != b.x ? a.x > b.x : a.y < b.y; });
    std::vector<int32_t> ids((size_t)count);
    for (int i = 0; i < count; ++i) ids[(size_t)i] = list[(size_t)i].y;
    if (count) {
        TRW_CUDA(cudaMalloc(&g->long_rows, sizeof(int32_t) * (size_t)count));
        TRW_CUDA(cudaMemcpy(g->long_rows, ids.data(), sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice));
    }
    g->n_long = count;
    return TRW_OK;
}

// Whether the edge weights are all >= 0 with a positive one in every
// non-empty row (checked once per graph).
int check_positive_rows(trw_graph *g, cudaStream_t st, bool &ok) {
    if (g->positive_rows == 0) {
        int *d_bad = nullptr;
        TRW_CUDA(cudaMalloc(&d_bad, sizeof(int)));
        TRW_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), st));
        TRW_CUDA(launch_positive_rows(dev_view(g), d_bad, st));
        int bad = 0;
        TRW_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        TRW_CUDA(cudaStreamSynchronize(st));
        cudaFree(d_bad);
        g->positive_rows = bad ? -1 : 1;
    }
    ok = g->positive_rows == 1;
    return TRW_OK;
}

int build_table(trw_graph *g, int sampler, int kind, cudaStream_t st) {
    const DevGraph d = dev_view(g);
    if (kind == TRW_WEIGHTS_EDGE && !g->weight) return fail(TRW_ERR_INVALID, "edge weights were not supplied");
    const int unit = kind == TRW_WEIGHTS_UNIT;
    // rebuilding a table in place: let walks still reading it (on any stream) finish
    if ((sampler == TRW_SAMPLER_ALIAS && g->alias) || (sampler == TRW_SAMPLER_ITS && g->prefix) ||
        (sampler == TRW_SAMPLER_REJECTION && g->rmax))
        TRW_CUDA(cudaDeviceSynchronize());
    if ((sampler == TRW_SAMPLER_ALIAS || sampler == TRW_SAMPLER_ITS) && g->n_long < 0) {
        int rc = collect_long_rows(g, st);
        if (rc) return rc;
    }
    if (sampler == TRW_SAMPLER_ALIAS) {
        if (!g->alias) TRW_CUDA(cudaMalloc(&g->alias, sizeof(AliasSlot) * (size_t)(g->e ? g->e : 1)));
        TRW_CUDA(launch_build_alias(d, unit, g->alias, g->long_rows, g->n_long, st));
        g->alias_kind = kind;
    } else if (sampler == TRW_SAMPLER_ITS) {
        if (!g->prefix) TRW_CUDA(cudaMalloc(&g->prefix, sizeof(double) * (size_t)(g->e ? g->e : 1)));
        TRW_CUDA(launch_build_prefix(d, unit, g->prefix, g->long_rows, g->n_long, st));
        g->prefix_kind = kind;
    } else if (sampler == TRW_SAMPLER_REJECTION) {
        if (!g->rmax) TRW_CUDA(cudaMalloc(&g->rmax, sizeof(double) * (size_t)g->n));
        TRW_CUDA(launch_build_max(d, unit, g->rmax, st));
        g->rmax_kind = kind;
    } else {
        return fail(TRW_ERR_INVALID, "sampler %d has no static table", sampler);
    }
    TRW_CUDA(cudaEventRecord(g->tables_done, st));
    return TRW_OK;
}

// Call-local plan: which kernel family and template arguments run.
struct Plan {
    bool warp_family = false;
    int sampler = kUniform;
    int update = kFixedLength;
    int weight_kind = kUnitWeight;
    int table_kind = -1;  // static table weights the run needs
};

// The walk's schema, if it names each label at most once (the label an
// edge carries then fixes the label the next step wants): next[l] for every
// label l < K, -1 where l is not in the schema or the label after it has no
// edges.
bool schema_next(const trw_walk_desc *d, int32_t K, LabelNext &next, std::vector<int32_t> &schema) {
    schema.assign(d->schema, d->schema + std::max(0, d->schema_len));
    if (schema.empty()) return false;
    for (int32_t l = 0; l < kMaxIndexedLabels; ++l) next.label[l] = -1;
    for (size_t i = 0; i < schema.size(); ++i) {
        const int32_t l = schema[i];
        for (size_t j = 0; j < i; ++j)
            if (schema[j] == l) return false;
        const int32_t w = schema[(i + 1) % schema.size()];
        if (l >= 0 && l < K) next.label[l] = (w >= 0 && w < K) ? w : -1;
    }
    return true;
}

// Builds (or rebuilds, for another schema) DevGraph::lab_fat when the label
// offsets (4 (K + 1) bytes per vertex) outgrow half the L2, so that their
// read is DRAM traffic: a step then reads one 16-byte entry instead of its
// block's positions and then the neighbour.  TRW_FAT_ADJACENCY=1 / 0 forces
// it on / off.  Waits for the device before overwriting an index that an
// earlier walk on any stream may still read.
int prepare_lab_fat(trw_graph *g, const trw_walk_desc *desc, cudaStream_t st) {
    if (g->lab_state != 1 || g->e <= 0) return TRW_OK;
    LabelNext next;
    std::vector<int32_t> schema;
    if (!schema_next(desc, g->lab_k, next, schema)) return TRW_OK;
    if (g->lab_fat_state == 1 && schema == g->lab_fat_schema) return TRW_OK;
    if (g->lab_fat_state == 0) {
        const char *force = getenv("TRW_FAT_ADJACENCY");
        int l2 = 0;
        TRW_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, g->device));
        const size_t off_bytes = sizeof(int32_t) * (size_t)g->n * (size_t)(g->lab_k + 1);
        const bool want = force && *force ? *force == '1' : off_bytes > (size_t)l2 / 2;
        const size_t bytes = sizeof(int4) * (size_t)g->e;
        size_t free_b = 0, total_b = 0;
        TRW_CUDA(cudaMemGetInfo(&free_b, &total_b));
        if (!want || bytes + (size_t(1) << 30) > free_b || cudaMalloc(&g->lab_fat, bytes) != cudaSuccess) {
            cudaGetLastError();
            g->lab_fat = nullptr;
            g->lab_fat_state = -1;
            return TRW_OK;
        }
    } else if (g->lab_fat_state == 1) {
        TRW_CUDA(cudaDeviceSynchronize());  // another schema's walks may still read it
        g->lab_fat_state = 0;
    } else {
        return TRW_OK;  // decided against
    }
    TRW_CUDA(launch_build_lab_fat(dev_view(g), next, g->lab_fat, st));
    TRW_CUDA(cudaStreamSynchronize(st));
    g->lab_fat_schema = schema;
    g->lab_fat_state = 1;
    return TRW_OK;
}

// DevGraph::lab_fat for a walk with this schema, or null.
const int4 *lab_fat_for(const trw_graph *g, const trw_walk_desc *desc) {
    if (g->lab_fat_state != 1) return nullptr;
    const std::vector<int32_t> schema(desc->schema, desc->schema + std::max(0, desc->schema_len));
    return schema == g->lab_fat_schema ? g->lab_fat : nullptr;
}

int make_plan(const trw_graph *g, const trw_walk_desc *d, Plan &pl) {
    if (d->app < 0 || d->app > 4) return fail(TRW_ERR_INVALID, "unknown app %d", d->app);
    pl.update = d->app == TRW_APP_PPR ? kGeometric : kFixedLength;
    // length_ starts at 1 and is compared with l_ only after a move, so l_ < 2
    // never ends (deepwalk.cpp:23-25); tp <= 0 never ends a PPR walk.
    if (pl.update == kFixedLength && d->length < 2) return fail(TRW_ERR_INVALID, "walk length must be >= 2");
    if (pl.update == kGeometric && !(d->tp >= 1e-6 && d->tp <= 1.0))
        return fail(TRW_ERR_INVALID, "PPR termination probability must be in [1e-6, 1]");
    if (d->app == TRW_APP_NODE2VEC && !(d->p > 0.0 && d->q > 0.0))
        return fail(TRW_ERR_INVALID, "Node2Vec p and q must be positive");
    const int wk = app_weight_kind(d->app);
    if (d->app == TRW_APP_METAPATH) {
        if (!g->label) return fail(TRW_ERR_INVALID, "MetaPath needs edge labels");
        if (!d->schema || d->schema_len < 1 || d->schema_len > TRW_MAX_SCHEMA)
            return fail(TRW_ERR_INVALID, "MetaPath schema length must be in [1, %d]", TRW_MAX_SCHEMA);
    }
    if (d->app == TRW_APP_NODE2VEC && !g->sorted)
        return fail(TRW_ERR_GRAPH, "Node2Vec needs sorted neighbour lists (Graph::is_neighbor)");
    switch (d->mode) {
    case TRW_MODE_UNIFORM:  // uniform_compute ignores the sampler (creeper.h:780-782)
        pl.sampler = kUniform;
        return TRW_OK;
    case TRW_MODE_STATIC:
        if (d->app == TRW_APP_NODE2VEC || d->app == TRW_APP_METAPATH)
            return fail(TRW_ERR_UNSUPPORTED, "static tables need walker-independent weights "
                                             "(the reference gathers them with an uninitialised walker)");
        if (d->sampler != TRW_SAMPLER_ITS && d->sampler != TRW_SAMPLER_ALIAS && d->sampler != TRW_SAMPLER_REJECTION)
            return fail(TRW_ERR_UNSUPPORTED, "static mode supports ITS, alias and rejection sampling");
        pl.sampler = d->sampler;
        pl.table_kind = d->app == TRW_APP_PPR ? TRW_WEIGHTS_UNIT : TRW_WEIGHTS_EDGE;
        if (pl.table_kind == TRW_WEIGHTS_EDGE && !g->weight) return fail(TRW_ERR_INVALID, "app needs edge weights");
        return TRW_OK;
    case TRW_MODE_DYNAMIC:
        if (wk == kEdgeWeight && !g->weight) return fail(TRW_ERR_INVALID, "app needs edge weights");
        pl.weight_kind = wk;
        if (d->sampler == TRW_SAMPLER_MAXWEIGHT_REJECTION) {
            if (d->app == TRW_APP_METAPATH)
                return fail(TRW_ERR_UNSUPPORTED, "MetaPath with max-weight rejection never terminates on "
                                                 "rows without a matching label");
            pl.sampler = kMaxRejection;
            return TRW_OK;
        }
        if (d->sampler == TRW_SAMPLER_ITS || d->sampler == TRW_SAMPLER_ALIAS || d->sampler == TRW_SAMPLER_REJECTION) {
            pl.warp_family = true;
            pl.sampler = d->sampler;
            return TRW_OK;
        }
        return fail(TRW_ERR_UNSUPPORTED, "dynamic mode supports ITS, alias, rejection and max-weight rejection");
    }
    return fail(TRW_ERR_INVALID, "unknown mode %d", d->mode);
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Largest u in [0, 2^32) with real2(u) * m = RN(u * 2^-32 * m) <= w (the
// max-weight rejection test), for m, w >= 0: the product is monotonic in u,
// so the device accepts a draw by comparing it with this integer.
uint32_t accept_threshold(double m, double w) {
    uint64_t lo = 0, hi = 0xffffffffull;  // u = 0 gives 0 <= w
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo + 1) / 2;
        volatile double r = (double)mid * (1.0 / 4294967296.0);
        volatile double y = r * m;
        if (y <= w) lo = mid; else hi = mid - 1;
    }
    return (uint32_t)lo;
}

// Largest v in [0, 2^32) with real1(v) = RN(v * RN(1 / (2^32 - 1))) <= t, for
// t >= 0.  real1 is monotonic in v, so the device compares the draw with
// this integer instead of converting it (same product, same rounding).
uint32_t real1_threshold(double t) {
    const double c = 1.0 / 4294967295.0;
    uint64_t lo = 0, hi = 0xffffffffull;  // real1(lo) <= t holds for t >= 0
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo + 1) / 2;
        volatile double r = (double)mid * c;
        if (r <= t) lo = mid; else hi = mid - 1;
    }
    return (uint32_t)lo;
}

// The app's hook parameters and the integer forms of its acceptance tests.
void fill_app_params(WalkParams &p, const trw_walk_desc *desc) {
    p.length = desc->length;
    p.schema_len = desc->app == TRW_APP_METAPATH ? desc->schema_len : 1;
    if (desc->app == TRW_APP_METAPATH)
        for (int i = 0; i < desc->schema_len; ++i) p.schema[i] = desc->schema[i];
    // node2vec.cpp:176-178,227,234: weights 1/p (return), 1 (common neighbour), 1/q
    p.p_w = desc->p != 0.0 ? 1.0 / desc->p : 0.0;
    p.q_w = desc->q != 0.0 ? 1.0 / desc->q : 0.0;
    p.n2v_max = std::max(1.0, std::max(p.q_w, p.p_w));
    // max_weight hooks: node2vec.cpp:198-205, ppr.cpp/metapath.cpp 1, deepwalk/genericwalk 5
    p.max_weight = desc->app == TRW_APP_NODE2VEC ? p.n2v_max
                 : (desc->app == TRW_APP_PPR || desc->app == TRW_APP_METAPATH) ? 1.0 : 5.0;
    p.tp = desc->tp;
    p.tp_max = real1_threshold(desc->tp);
    const double w[4] = {p.n2v_max, p.p_w, 1.0, p.q_w};  // n2v_class order; [2] is PPR's unit weight
    for (int k = 0; k < 4; ++k) p.accept_max[k] = accept_threshold(p.max_weight, w[k]);
    p.seed = desc->seed;
}

// Streams, events and pinned words of the host-output pipelines (created on
// first use).
int ensure_host_pipeline(trw_graph *g) {
    if (!g->copy_stream) TRW_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    if (!g->aux_stream) TRW_CUDA(cudaStreamCreateWithFlags(&g->aux_stream, cudaStreamNonBlocking));
    if (!g->h_ends) TRW_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&g->h_ends), sizeof(int64_t) * kMaxRanges,
                                           cudaHostAllocDefault));
    for (cudaEvent_t *e : {&g->ev_fork, &g->ev_join})
        if (!*e) TRW_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (int r = 0; r < kMaxRanges; ++r) {
        if (!g->range_done[r]) TRW_CUDA(cudaEventCreateWithFlags(&g->range_done[r], cudaEventDisableTiming));
        if (!g->offsets_done[r]) TRW_CUDA(cudaEventCreateWithFlags(&g->offsets_done[r], cudaEventDisableTiming));
    }
    return TRW_OK;
}

// The kernel a walk runs and the graph structures it needs, built on first
// use (the caller holds the graph lock and has made the device current).
int prepare_plan(trw_graph *g, const trw_walk_desc *desc, Plan &pl, cudaStream_t st) {
    int rc = TRW_OK;
    // Dynamic mode with walker-independent weights (DeepWalk and GenericWalk:
    // edge weights; PPR: 1) gathers the same row every step, so its per-step
    // ITS prefix, alias table or row maximum is the static one (same builder
    // arithmetic in the same order, same draws): such walks run on the static
    // tables.  Dynamic alias and rejection stop a walker on a row without a
    // positive weight where the static forms move it, so they map only when
    // the graph has no such row.
    if (pl.warp_family && (pl.weight_kind == kEdgeWeight || pl.weight_kind == kUnitWeight) &&
        (pl.sampler == kITS || pl.sampler == kAlias || pl.sampler == kRejection)) {
        const int kind = pl.weight_kind == kUnitWeight ? TRW_WEIGHTS_UNIT : TRW_WEIGHTS_EDGE;
        bool same = pl.sampler == kITS || kind == TRW_WEIGHTS_UNIT;
        if (!same) {
            rc = check_positive_rows(g, st, same);
            if (rc) return rc;
        }
        if (same) {
            pl.warp_family = false;
            pl.table_kind = kind;
        }
    }
    if (pl.table_kind >= 0) {
        const int have = pl.sampler == kAlias ? g->alias_kind : pl.sampler == kITS ? g->prefix_kind : g->rmax_kind;
        if (have != pl.table_kind) {  // compute() rebuilds its static tables each run (creeper.h:700-702)
            rc = build_table(g, pl.sampler, pl.table_kind, st);
            if (rc) return rc;
        }
        TRW_CUDA(cudaStreamWaitEvent(st, g->tables_done, 0));  // built on another stream, perhaps
    }

    if (desc->app == TRW_APP_NODE2VEC && g->edge_state == 0) {
        rc = build_edge_set(g, st);
        if (rc) return rc;
    }
    if (!pl.warp_family && (pl.sampler == kUniform || pl.sampler == kMaxRejection) && g->fat_state == 0) {
        rc = build_fat_adjacency(g, st);
        if (rc) return rc;
    }
    if (desc->app == TRW_APP_METAPATH && pl.warp_family && pl.sampler == kITS) {
        if (g->lab_state == 0) {
            rc = build_label_index(g, st);
            if (rc) return rc;
        }
        if (g->lab_state == 1) {  // the thread engine answers from the label index
            pl.warp_family = false;
            pl.sampler = kLabelIndex;
        }
    }

    return TRW_OK;
}

// Shared implementation of trw_walk and trw_ppr_batch.
int run_walk(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_sources,
             int64_t num_walkers, int64_t per_query, int64_t id_base, int32_t *paths, int32_t path_cap,
             int32_t *lengths, int32_t *counts, int64_t counts_len, bool zero_counts, uint64_t *steps,
             int32_t engine, cudaStream_t st, int32_t *table = nullptr, int32_t table_bits = 0,
             bool hold_lock = false) {
    if (!g || !desc) return fail(TRW_ERR_INVALID, "null graph or descriptor");
    if (num_walkers < 0 || (num_walkers > 0 && !sources)) return fail(TRW_ERR_INVALID, "bad walker arguments");
    if (paths && path_cap <= 0) return fail(TRW_ERR_INVALID, "path_cap must be > 0 when paths are requested");
    if (engine != TRW_ENGINE_PERSISTENT && engine != TRW_ENGINE_PLAIN) return fail(TRW_ERR_INVALID, "bad engine");
    Plan pl;
    int rc = make_plan(g, desc, pl);
    if (rc) return rc;
    std::unique_lock<std::mutex> lock(g->mu, std::defer_lock);
    if (!hold_lock) lock.lock();
    TRW_CUDA(cudaSetDevice(g->device));
    rc = prepare_plan(g, desc, pl, st);
    if (rc) return rc;
    if (pl.sampler == kLabelIndex) {
        rc = prepare_lab_fat(g, desc, st);
        if (rc) return rc;
    }

    // Stage host buffers.
    const bool h_src = sources && !is_device_ptr(sources);
    const bool h_paths = paths && !is_device_ptr(paths);
    const bool h_len = lengths && !is_device_ptr(lengths);
    const bool h_cnt = counts && !is_device_ptr(counts);
    const bool h_steps = steps && !is_device_ptr(steps);
    const size_t b_src = h_src ? align_up(sizeof(int32_t) * (size_t)num_sources) : 0;
    const size_t b_paths = h_paths ? align_up(sizeof(int32_t) * (size_t)num_walkers * (size_t)path_cap) : 0;
    const size_t b_len = h_len ? align_up(sizeof(int32_t) * (size_t)num_walkers) : 0;
    const size_t b_cnt = h_cnt ? align_up(sizeof(int32_t) * (size_t)counts_len) : 0;
    const bool staged = b_src || b_paths || b_len || b_cnt;
    if (staged) TRW_CUDA(g->stage.ensure(b_src + b_paths + b_len + b_cnt + 256));
    char *base = static_cast<char *>(g->stage.p);
    const int32_t *d_src = sources;
    int32_t *d_paths = paths, *d_len = lengths, *d_cnt = counts;
    if (h_src) {
        d_src = reinterpret_cast<int32_t *>(base);
        TRW_CUDA(cudaMemcpyAsync((void *)d_src, sources, sizeof(int32_t) * num_sources, cudaMemcpyHostToDevice, st));
    }
    base += b_src;
    if (h_paths) d_paths = reinterpret_cast<int32_t *>(base);
    base += b_paths;
    if (h_len) d_len = reinterpret_cast<int32_t *>(base);
    base += b_len;
    if (h_cnt) {
        d_cnt = reinterpret_cast<int32_t *>(base);
        if (zero_counts) TRW_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(int32_t) * counts_len, st));
        else TRW_CUDA(cudaMemcpyAsync(d_cnt, counts, sizeof(int32_t) * counts_len, cudaMemcpyHostToDevice, st));
    } else if (counts && zero_counts) {
        TRW_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(int32_t) * counts_len, st));
    }

    // Engine state slot (queue head + step counter), reused after its event.
    EngineSlot &slot = g->slots[g->next_slot];
    g->next_slot = (g->next_slot + 1) % kEngineSlots;
    if (slot.used) TRW_CUDA(cudaEventSynchronize(slot.done));
    TRW_CUDA(cudaMemsetAsync(slot.queue_head, 0, 2 * sizeof(unsigned long long), st));

    WalkParams p;
    std::memset(&p, 0, sizeof p);
    p.g = dev_view(g);
    if (pl.sampler == kLabelIndex) p.g.lab_fat = lab_fat_for(g, desc);
    fill_app_params(p, desc);
    p.static_unit = pl.table_kind == TRW_WEIGHTS_UNIT;
    p.sources = d_src;
    p.num_walkers = num_walkers;
    p.per_query = per_query;
    p.id_base = id_base;
    p.paths = d_paths;
    p.path_cap = paths ? path_cap : 0;
    p.path_vec = d_paths && path_cap % 4 == 0 && reinterpret_cast<uintptr_t>(d_paths) % 16 == 0;
    p.lengths = d_len;
    p.counts = d_cnt;
    p.queue_head = slot.queue_head;
    p.steps = slot.steps;
    p.error = g->error;
    p.table = table;
    p.table_bits = table_bits;

    LaunchShape shape = g->shape[pl.sampler == kLabelIndex ? (int)kITS : pl.sampler];
    shape.engine = engine;
    shape.num_sms = g->num_sms;
    if (shape.ring < 0) {  // the shape set for this sampler is the plain form (one thread per walker)
        if (!pl.warp_family) shape.engine = kEnginePlain;
        shape.ring = 0;
    }
    if (shape.ring == 0) {
        // Automatic ring depth (launch-shape sweeps on GB300): one walker per
        // lane when visits go to sparse tables (their insert records cost
        // registers), for max-weight rejection (its trial loop and neighbour
        // search hold more state per walker: Node2Vec on R-MAT 2^24 with
        // paths takes 65.2 ms at one, 72.0 ms at two, 78 ms at four) and
        // when there are too few walkers to give every lane several; four
        // otherwise.
        const int64_t lanes = (int64_t)g->num_sms * 2048;
        shape.ring = (table || pl.sampler == kMaxRejection || num_walkers < 4 * lanes) ? 1 : 4;
    }
    cudaError_t le;
    if (g->profile) {
        TRW_CUDA(cudaEventRecord(g->ev_walk0, st));
        g->have_post = false;
    }
    if (pl.warp_family) {
        if (pl.sampler == kAlias) {
            // one raw + one table row of max_degree slots per warp, at most 1 GiB
            const int64_t stride = 2 * (int64_t)std::max(1, g->max_degree);
            int64_t warps = warp_engine_warps(p, shape);
            const int64_t cap = (int64_t)((1ull << 30) / (sizeof(AliasSlot) * (uint64_t)stride));
            if (warps > cap) warps = cap;
            warps = std::max<int64_t>(8, warps / 8 * 8);
            TRW_CUDA(g->alias_scratch.ensure(sizeof(AliasSlot) * (size_t)(warps * stride)));
            p.alias_scratch = static_cast<AliasSlot *>(g->alias_scratch.p);
            p.alias_scratch_stride = stride;
            shape.max_warps = warps;
            TRW_CUDA(cudaStreamWaitEvent(st, g->scratch_done, 0));
        }
        le = launch_walk_warp(p, pl.sampler, pl.update, pl.weight_kind, shape, st);
        if (le == cudaSuccess && pl.sampler == kAlias) le = cudaEventRecord(g->scratch_done, st);
    } else {
        le = launch_walk_thread(p, pl.sampler, pl.update, pl.weight_kind, shape, st);
    }
    if (le != cudaSuccess) return fail(TRW_ERR_CUDA, "walk launch: %s", cudaGetErrorString(le));
    if (g->profile) TRW_CUDA(cudaEventRecord(g->ev_walk1, st));
    if (steps) TRW_CUDA(cudaMemcpyAsync(steps, slot.steps, sizeof(uint64_t), h_steps ? cudaMemcpyDeviceToHost
                                                                                      : cudaMemcpyDeviceToDevice, st));
    if (h_paths) TRW_CUDA(cudaMemcpyAsync(paths, d_paths, sizeof(int32_t) * (size_t)num_walkers * path_cap,
                                          cudaMemcpyDeviceToHost, st));
    if (h_len) TRW_CUDA(cudaMemcpyAsync(lengths, d_len, sizeof(int32_t) * (size_t)num_walkers, cudaMemcpyDeviceToHost, st));
    if (h_cnt) TRW_CUDA(cudaMemcpyAsync(counts, d_cnt, sizeof(int32_t) * (size_t)counts_len, cudaMemcpyDeviceToHost, st));
    TRW_CUDA(cudaEventRecord(slot.done, st));
    slot.used = true;
    if (staged || h_steps) {
        TRW_CUDA(cudaStreamSynchronize(st));
        int err = 0;
        TRW_CUDA(cudaMemcpy(&err, g->error, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            TRW_CUDA(cudaMemset(g->error, 0, sizeof(int)));
            return fail(TRW_ERR_DEVICE, "device error word %d (1 = rejection trial limit, 2 = invalid source vertex)", err);
        }
    }
    return TRW_OK;
}

// trw_walk into host paths / lengths for a large batch: the walkers run as
// ranges alternating between two compute streams, and each range's paths
// and lengths are copied to the host on the copy stream while the next range
// walks (the pipeline of the sparse PPR batches).  Walker ids continue across
// ranges, so the walks are exactly those of one launch.  `taken` stays false
// (and nothing runs) when the batch has fewer than four walkers per lane of
// the GPU, or when the outputs are on the device.
int walk_host_ranges(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t W, int64_t id_base,
                     int32_t *paths, int32_t path_cap, int32_t *lengths, int32_t *counts, uint64_t *steps,
                     int32_t engine, cudaStream_t st, bool &taken) {
    taken = false;
    if (!g || !desc || W <= 0 || !sources || (paths && path_cap <= 0)) return TRW_OK;
    const bool h_paths = paths && !is_device_ptr(paths);
    const bool h_len = lengths && !is_device_ptr(lengths);
    if ((!h_paths && !h_len) || (paths && !h_paths) || (lengths && !h_len)) return TRW_OK;
    // One range per lane's worth of walkers, up to kMaxRanges (MetaPath on
    // R-MAT 2^24, 2^22 walkers, L = 20: 2.48 ms end to end with 13 ranges,
    // 2.70 ms with 6; more compute streams or uneven ranges did not help).
    const int64_t lanes = (int64_t)g->num_sms * 2048;
    const int64_t ranges = std::min<int64_t>(kMaxRanges, W / lanes);
    if (W < 4 * lanes || ranges < 2) return TRW_OK;
    taken = true;
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    int rc = ensure_host_pipeline(g);
    if (rc) return rc;
    const bool h_src = !is_device_ptr(sources);
    const bool h_cnt = counts && !is_device_ptr(counts);
    const bool h_steps = steps && !is_device_ptr(steps);
    const size_t b_src = h_src ? align_up(sizeof(int32_t) * (size_t)W) : 0;
    const size_t b_cnt = h_cnt ? align_up(sizeof(int32_t) * (size_t)g->n) : 0;
    TRW_CUDA(g->stage.ensure(b_src + b_cnt + sizeof(uint64_t) * (kMaxRanges + 1)));
    char *sb = static_cast<char *>(g->stage.p);
    const int32_t *d_src = h_src ? reinterpret_cast<const int32_t *>(sb) : sources;
    int32_t *d_cnt = h_cnt ? reinterpret_cast<int32_t *>(sb + b_src) : counts;
    uint64_t *d_steps = reinterpret_cast<uint64_t *>(sb + b_src + b_cnt);
    const size_t b_paths = paths ? align_up(sizeof(int32_t) * (size_t)W * (size_t)path_cap) : 0;
    TRW_CUDA(g->stage_out.ensure(b_paths + (lengths ? align_up(sizeof(int32_t) * (size_t)W) : 0) + 256));
    int32_t *d_paths = paths ? static_cast<int32_t *>(g->stage_out.p) : nullptr;
    int32_t *d_len = lengths ? reinterpret_cast<int32_t *>(static_cast<char *>(g->stage_out.p) + b_paths) : nullptr;
    if (h_src) TRW_CUDA(cudaMemcpyAsync((void *)d_src, sources, sizeof(int32_t) * (size_t)W, cudaMemcpyHostToDevice, st));
    // trw_walk adds to the caller's counts
    if (h_cnt) TRW_CUDA(cudaMemcpyAsync(d_cnt, counts, sizeof(int32_t) * (size_t)g->n, cudaMemcpyHostToDevice, st));
    TRW_CUDA(cudaEventRecord(g->ev_fork, st));
    TRW_CUDA(cudaStreamWaitEvent(g->aux_stream, g->ev_fork, 0));
    const cudaStream_t rs[2] = {st, g->aux_stream};
    const int64_t per = (W + ranges - 1) / ranges;
    int nr = 0;
    for (int64_t ws = 0; ws < W; ws += per, ++nr) {
        const int64_t n = std::min(per, W - ws);
        rc = run_walk(g, desc, d_src + ws, n, n, 0, id_base + ws, d_paths ? d_paths + ws * path_cap : nullptr,
                      path_cap, d_len ? d_len + ws : nullptr, d_cnt, counts ? (int64_t)g->n : 0, false, d_steps + nr,
                      engine, rs[nr & 1], nullptr, 0, /*hold_lock=*/true);
        if (rc) {
            // ranges already queued still write the staging buffers: let them finish before returning
            cudaStreamSynchronize(g->aux_stream);
            cudaStreamSynchronize(st);
            return rc;
        }
        TRW_CUDA(cudaEventRecord(g->range_done[nr], rs[nr & 1]));
    }
    TRW_CUDA(cudaEventRecord(g->ev_join, g->aux_stream));
    TRW_CUDA(cudaStreamWaitEvent(st, g->ev_join, 0));
    if (steps) {
        uint64_t *sum = h_steps ? d_steps + kMaxRanges : steps;
        TRW_CUDA(launch_sum_steps(d_steps, nr, sum, st));
        if (h_steps) TRW_CUDA(cudaMemcpyAsync(steps, sum, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    }
    if (h_cnt) TRW_CUDA(cudaMemcpyAsync(counts, d_cnt, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, st));
    int64_t ws = 0;
    for (int r = 0; r < nr; ++r, ws += per) {
        const int64_t n = std::min(per, W - ws);
        TRW_CUDA(cudaEventSynchronize(g->range_done[r]));
        if (paths) TRW_CUDA(cudaMemcpyAsync(paths + ws * path_cap, d_paths + ws * path_cap,
                                            sizeof(int32_t) * (size_t)n * (size_t)path_cap, cudaMemcpyDeviceToHost,
                                            g->copy_stream));
        if (lengths) TRW_CUDA(cudaMemcpyAsync(lengths + ws, d_len + ws, sizeof(int32_t) * (size_t)n,
                                              cudaMemcpyDeviceToHost, g->copy_stream));
    }
    TRW_CUDA(cudaStreamSynchronize(st));
    TRW_CUDA(cudaStreamSynchronize(g->copy_stream));
    int err = 0;
    TRW_CUDA(cudaMemcpy(&err, g->error, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        TRW_CUDA(cudaMemset(g->error, 0, sizeof(int)));
        return fail(TRW_ERR_DEVICE, "device error word %d (1 = rejection trial limit, 2 = invalid source vertex)", err);
    }
    return TRW_OK;
}

}  // namespace

extern "C" {

int32_t trw_version(void) { return 1000; }

const char *trw_last_error(void) { return g_last_error.c_str(); }

int trw_graph_create(const int64_t *row_ptr, const int32_t *adj, const double *weight, const int32_t *label,
                     int32_t n, int64_t e, uint32_t flags, trw_graph **out) {
    if (!out) return fail(TRW_ERR_INVALID, "out is null");
    *out = nullptr;
    if (n <= 0 || e < 0 || !row_ptr || (e > 0 && !adj)) return fail(TRW_ERR_INVALID, "bad CSR arguments");
    if (e >= (int64_t)1 << 31) return fail(TRW_ERR_CAPACITY, "e = %lld: the library stores int32 row offsets (e < 2^31)",
                                           (long long)e);
    trw_graph *g = new trw_graph();
    auto bail = [&](int code) { destroy_graph(g); return code; };
    if (cudaGetDevice(&g->device) != cudaSuccess) return bail(fail(TRW_ERR_CUDA, "no CUDA device"));
    cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device);
    g->n = n;
    g->e = e;
    {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, g->device);
        g->adj_streams = l2 > 0 && sizeof(int32_t) * (size_t)e >= 2 * (size_t)l2;
    }
    const size_t es = (size_t)(e ? e : 1);
    int64_t *d_row = nullptr;
    int *d_flags = nullptr;
    cudaError_t ce = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (ce == cudaSuccess) ce = x; };
    chk(cudaMalloc(&g->rows, sizeof(int2) * (size_t)n));
    chk(cudaMalloc(&g->adj, sizeof(int32_t) * es));
    chk(cudaMalloc(&d_row, sizeof(int64_t) * ((size_t)n + 1)));
    chk(cudaMalloc(&d_flags, 3 * sizeof(int)));
    if (weight) chk(cudaMalloc(&g->weight, sizeof(double) * es));
    // labels padded to a multiple of 4 elements: the label ITS reads aligned 16-byte words
    const size_t es4 = (es + 3) & ~(size_t)3;
    if (label) chk(cudaMalloc(&g->label, sizeof(int32_t) * es4));
    if (label) chk(cudaMemset(g->label, 0, sizeof(int32_t) * es4));
    chk(cudaMalloc(&g->state, sizeof(unsigned long long) * (2 * kEngineSlots + 1)));
    if (ce != cudaSuccess) { cudaFree(d_row); cudaFree(d_flags); return bail(fail(TRW_ERR_CUDA, "graph allocation: %s", cudaGetErrorString(ce))); }
    g->error = reinterpret_cast<int *>(g->state + 2 * kEngineSlots);
    for (int i = 0; i < kEngineSlots; ++i) {
        g->slots[i].queue_head = g->state + 2 * i;
        g->slots[i].steps = g->state + 2 * i + 1;
        chk(cudaEventCreateWithFlags(&g->slots[i].done, cudaEventDisableTiming));
    }
    chk(cudaEventCreateWithFlags(&g->scratch_done, cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&g->ppr_done, cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&g->tables_done, cudaEventDisableTiming));
    chk(cudaMemset(g->state, 0, sizeof(unsigned long long) * (2 * kEngineSlots + 1)));
    chk(cudaMemcpy(d_row, row_ptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDefault));
    if (e) chk(cudaMemcpy(g->adj, adj, sizeof(int32_t) * (size_t)e, cudaMemcpyDefault));
    if (weight && e) chk(cudaMemcpy(g->weight, weight, sizeof(double) * (size_t)e, cudaMemcpyDefault));
    if (label && e) chk(cudaMemcpy(g->label, label, sizeof(int32_t) * (size_t)e, cudaMemcpyDefault));
    chk(cudaMemset(d_flags, 0, 3 * sizeof(int)));
    // pass 1 without the sortedness check decides validity; pass 2 records sortedness
    if (ce == cudaSuccess) ce = launch_validate_graph(d_row, g->adj, n, e, 0, g->rows, d_flags, d_flags + 1, 0);
    if (ce == cudaSuccess) ce = launch_validate_graph(d_row, g->adj, n, e, 1, g->rows, d_flags + 2, d_flags + 1, 0);
    int hf[3] = {0, 0, 0};
    chk(cudaMemcpy(hf, d_flags, sizeof hf, cudaMemcpyDeviceToHost));
    cudaFree(d_row);
    cudaFree(d_flags);
    if (ce != cudaSuccess) return bail(fail(TRW_ERR_CUDA, "graph upload: %s", cudaGetErrorString(ce)));
    if (hf[0]) return bail(fail(TRW_ERR_GRAPH, "invalid CSR (flags %d: 1 offsets, 2 monotonicity, 4 vertex id range)", hf[0]));
    g->sorted = (hf[2] & 8) == 0;
    if ((flags & TRW_GRAPH_CHECK_SORTED) && !g->sorted) return bail(fail(TRW_ERR_GRAPH, "neighbour lists are not sorted"));
    g->max_degree = hf[1];
    *out = g;
    return TRW_OK;
}

int trw_graph_destroy(trw_graph *g) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    cudaSetDevice(g->device);
    cudaDeviceSynchronize();
    destroy_graph(g);
    return TRW_OK;
}

int trw_graph_info(const trw_graph *g, int32_t *n, int64_t *e, int32_t *max_degree) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    if (n) *n = g->n;
    if (e) *e = g->e;
    if (max_degree) *max_degree = g->max_degree;
    return TRW_OK;
}

int trw_graph_indexes(const trw_graph *g, int32_t *edge_set_state, int32_t *label_index_state) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    if (edge_set_state) *edge_set_state = g->edge_state;
    if (label_index_state) *label_index_state = g->lab_state;
    return TRW_OK;
}

int trw_graph_layout(const trw_graph *g, int32_t *fat_adjacency_state, int32_t *fat_label_index_state) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    if (fat_adjacency_state) *fat_adjacency_state = g->fat_state;
    if (fat_label_index_state) *fat_label_index_state = g->lab_fat_state;
    return TRW_OK;
}

int trw_graph_build_indexes(trw_graph *g, int32_t edge_set, int32_t label_index, trw_stream_t stream) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (edge_set) {
        int rc = build_edge_set(g, st);
        if (rc) return rc;
        rc = build_fat_adjacency(g, st);  // decided by the same rule as in a walk
        if (rc) return rc;
    }
    if (label_index) {
        const int rc = build_label_index(g, st);
        if (rc) return rc;
    }
    TRW_CUDA(cudaStreamSynchronize(st));
    return TRW_OK;
}

int trw_graph_synchronize(trw_graph *g) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    TRW_CUDA(cudaSetDevice(g->device));
    TRW_CUDA(cudaDeviceSynchronize());
    return TRW_OK;
}

int trw_tables_build(trw_graph *g, int32_t sampler, int32_t weight_kind, trw_stream_t stream) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    if (weight_kind != TRW_WEIGHTS_EDGE && weight_kind != TRW_WEIGHTS_UNIT) return fail(TRW_ERR_INVALID, "bad weight kind");
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    return build_table(g, sampler, weight_kind, reinterpret_cast<cudaStream_t>(stream));
}

int trw_tables_download(const trw_graph *g, int32_t sampler, void *out, size_t out_bytes) {
    if (!g || !out) return fail(TRW_ERR_INVALID, "null argument");
    const void *src = nullptr;
    size_t bytes = 0;
    if (sampler == TRW_SAMPLER_ALIAS) { src = g->alias; bytes = sizeof(AliasSlot) * (size_t)g->e; }
    else if (sampler == TRW_SAMPLER_ITS) { src = g->prefix; bytes = sizeof(double) * (size_t)g->e; }
    else if (sampler == TRW_SAMPLER_REJECTION) { src = g->rmax; bytes = sizeof(double) * (size_t)g->n; }
    else return fail(TRW_ERR_INVALID, "sampler %d has no static table", sampler);
    if (!src) return fail(TRW_ERR_NO_TABLES, "table not built");
    if (out_bytes < bytes) return fail(TRW_ERR_CAPACITY, "output holds %zu bytes, table needs %zu", out_bytes, bytes);
    TRW_CUDA(cudaSetDevice(g->device));
    TRW_CUDA(cudaDeviceSynchronize());
    TRW_CUDA(cudaMemcpy(out, src, bytes, cudaMemcpyDefault));
    return TRW_OK;
}

int trw_tables_upload(trw_graph *g, int32_t sampler, int32_t weight_kind, const void *table, size_t bytes,
                      trw_stream_t stream) {
    if (!g || !table) return fail(TRW_ERR_INVALID, "null argument");
    if (weight_kind != TRW_WEIGHTS_EDGE && weight_kind != TRW_WEIGHTS_UNIT) return fail(TRW_ERR_INVALID, "bad weight kind");
    size_t want = 0;
    if (sampler == TRW_SAMPLER_ALIAS) want = sizeof(AliasSlot) * (size_t)g->e;
    else if (sampler == TRW_SAMPLER_ITS) want = sizeof(double) * (size_t)g->e;
    else if (sampler == TRW_SAMPLER_REJECTION) want = sizeof(double) * (size_t)g->n;
    else return fail(TRW_ERR_INVALID, "sampler %d has no static table", sampler);
    if (bytes != want) return fail(TRW_ERR_INVALID, "table holds %zu bytes, this graph's needs %zu", bytes, want);
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    void **dst = sampler == TRW_SAMPLER_ALIAS ? reinterpret_cast<void **>(&g->alias)
               : sampler == TRW_SAMPLER_ITS ? reinterpret_cast<void **>(&g->prefix)
                                            : reinterpret_cast<void **>(&g->rmax);
    if (*dst) TRW_CUDA(cudaDeviceSynchronize());  // walks on any stream may still read the old table
    else TRW_CUDA(cudaMalloc(dst, std::max<size_t>(want, 16)));
    if (want) TRW_CUDA(cudaMemcpyAsync(*dst, table, want, cudaMemcpyDefault, st));
    if (sampler == TRW_SAMPLER_ALIAS) g->alias_kind = weight_kind;
    else if (sampler == TRW_SAMPLER_ITS) g->prefix_kind = weight_kind;
    else g->rmax_kind = weight_kind;
    TRW_CUDA(cudaEventRecord(g->tables_done, st));
    TRW_CUDA(cudaStreamSynchronize(st));  // the caller may free or reuse `table` on return
    return TRW_OK;
}

int trw_walk(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_walkers, int64_t id_base,
             int32_t *paths, int32_t path_cap, int32_t *lengths, int32_t *counts, uint64_t *steps, int32_t engine,
             trw_stream_t stream) {
    bool taken = false;
    const int rc = walk_host_ranges(g, desc, sources, num_walkers, id_base, paths, path_cap, lengths, counts, steps,
                                    engine, reinterpret_cast<cudaStream_t>(stream), taken);
    if (taken) return rc;
    return run_walk(g, desc, sources, num_walkers, num_walkers, 0, id_base, paths, path_cap, lengths, counts,
                    g ? (int64_t)g->n : 0, false, steps, engine, reinterpret_cast<cudaStream_t>(stream));
}

int trw_ppr_batch(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_queries,
                  int64_t walkers_per_query, int32_t *counts, uint64_t *steps, uint32_t flags, int32_t engine,
                  trw_stream_t stream) {
    if (!g || !desc) return fail(TRW_ERR_INVALID, "null graph or descriptor");
    if (num_queries < 0 || walkers_per_query <= 0) return fail(TRW_ERR_INVALID, "bad batch shape");
    if (desc->app != TRW_APP_PPR) return fail(TRW_ERR_INVALID, "trw_ppr_batch runs the PPR app");
    return run_walk(g, desc, sources, num_queries, num_queries * walkers_per_query, walkers_per_query, 0, nullptr, 0,
                    nullptr, counts, num_queries * (int64_t)g->n, (flags & TRW_PPR_ZERO_COUNTS) != 0, steps, engine,
                    reinterpret_cast<cudaStream_t>(stream));
}

int trw_ppr_batch_sparse(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_queries,
                         int64_t walkers_per_query, int64_t *offsets, int32_t *vertices, int32_t *counts,
                         int64_t capacity, uint64_t *steps, int32_t engine, trw_stream_t stream) {
    if (!g || !desc) return fail(TRW_ERR_INVALID, "null graph or descriptor");
    if (num_queries < 0 || walkers_per_query <= 0) return fail(TRW_ERR_INVALID, "bad batch shape");
    if (desc->app != TRW_APP_PPR) return fail(TRW_ERR_INVALID, "trw_ppr_batch_sparse runs the PPR app");
    if (!offsets || capacity < 0 || (capacity > 0 && (!vertices || !counts)))
        return fail(TRW_ERR_INVALID, "offsets and (vertices, counts) of `capacity` entries are required");
    if (!(desc->tp >= 1e-6 && desc->tp <= 1.0)) return fail(TRW_ERR_INVALID, "PPR termination probability must be in [1e-6, 1]");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    // The tables (and counters) are shared by every sparse batch on this
    // graph: calls on different streams run one after the other on the device.
    TRW_CUDA(cudaStreamWaitEvent(st, g->ppr_done, 0));
    // Table size: 2^bits >= 1.25 x the expected visits of a query (walkers /
    // tp), which bounds its distinct vertices, and never above 2 x the vertex
    // count (a query cannot visit more).
    const double visits = (double)walkers_per_query / desc->tp;
    int32_t bits = 10;
    while (bits < 30 && (double)(1ll << bits) < 1.25 * visits) ++bits;
    while (bits > 10 && (1ll << (bits - 1)) >= 2ll * g->n) --bits;
    if (num_queries > 0 && (g->ppr_bits != bits || g->ppr_queries < num_queries || g->ppr_dirty)) {
        const size_t bytes = sizeof(int2) * ((size_t)num_queries << bits);
        TRW_CUDA(g->ppr_tables.ensure(bytes));
        TRW_CUDA(cudaMemsetAsync(g->ppr_tables.p, 0, bytes, st));
        g->ppr_bits = bits;
        g->ppr_queries = num_queries;
    }
    // staging for host buffers: sources in; offsets, vertices, counts out
    const bool h_src = num_queries > 0 && !is_device_ptr(sources);
    const bool h_off = !is_device_ptr(offsets);
    const bool h_v = vertices && !is_device_ptr(vertices);
    const bool h_c = counts && !is_device_ptr(counts);
    const bool h_steps = steps && !is_device_ptr(steps);
    const bool host_out = h_off || h_v || h_c;
    // With host outputs the batch runs as ranges of queries (below), each
    // post-processed while the next range walks; smaller post-processing
    // chunks keep one range's emit from running as a single long wave.
    const int32_t cbits = host_out ? kPprRangeChunkBits : kPprChunkBits;
    const int64_t dist_ints = ppr_distinct_ints(bits, cbits);  // per query: total + segment prefixes
    const size_t b_dist = align_up(sizeof(int32_t) * (size_t)dist_ints * (size_t)std::max<int64_t>(1, num_queries));
    TRW_CUDA(g->ppr_distinct.ensure(b_dist + sizeof(uint64_t) * (kMaxRanges + 1)));
    int32_t *tables = static_cast<int32_t *>(g->ppr_tables.p);
    int32_t *distinct = static_cast<int32_t *>(g->ppr_distinct.p);
    uint64_t *d_steps = reinterpret_cast<uint64_t *>(static_cast<char *>(g->ppr_distinct.p) + b_dist);

    const size_t b_src = h_src ? align_up(sizeof(int32_t) * (size_t)num_queries) : 0;
    if (h_src) TRW_CUDA(g->stage.ensure(b_src));
    const size_t b_off = h_off ? align_up(sizeof(int64_t) * (size_t)(num_queries + 1)) : 0;
    const size_t b_v = h_v ? align_up(sizeof(int32_t) * (size_t)capacity) : 0;
    const size_t b_c = h_c ? align_up(sizeof(int32_t) * (size_t)capacity) : 0;
    if (b_off + b_v + b_c) TRW_CUDA(g->stage_out.ensure(b_off + b_v + b_c + 256));
    char *ob = static_cast<char *>(g->stage_out.p);
    int64_t *d_off = h_off ? reinterpret_cast<int64_t *>(ob) : offsets;
    int32_t *d_v = h_v ? reinterpret_cast<int32_t *>(ob + b_off) : vertices;
    int32_t *d_c = h_c ? reinterpret_cast<int32_t *>(ob + b_off + b_v) : counts;
    const int32_t *d_src = sources;
    if (h_src) {
        d_src = static_cast<const int32_t *>(g->stage.p);
        TRW_CUDA(cudaMemcpyAsync((void *)d_src, sources, sizeof(int32_t) * (size_t)num_queries,
                                 cudaMemcpyHostToDevice, st));
    }

    // With host outputs the batch runs as several ranges of queries (split
    // by kPprSplit, or up to kPprRanges equal ones): while one range walks,
    // the copy stream moves the previous range's entries to the host (a
    // device-to-host copy runs at about half the rate the entries are
    // produced, so it hides behind the next walk).  Ranges
    // alternate between two compute streams so that the next range's walk
    // fills the GPU while the last walkers of a range finish; only the
    // offsets scans are chained across ranges.  Every range keeps at least 8
    // walkers per lane of the GPU.  bounds[r] .. bounds[r + 1] = range r.
    std::vector<int64_t> bounds{0};
    if (host_out && num_queries > 1) {
        const int64_t lanes = (int64_t)g->num_sms * 2048;
        const int64_t by_walkers = num_queries * walkers_per_query / (8 * lanes);
        if (by_walkers >= kPprSplitUnits && num_queries >= 2 * kPprSplitUnits) {
            int64_t acc = 0;
            for (int w : kPprSplit) {
                acc += w;
                bounds.push_back(num_queries * acc / kPprSplitUnits);
            }
        } else {
            const int64_t n = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(kPprRanges, num_queries),
                                                                     by_walkers));
            const int64_t per = (num_queries + n - 1) / n;
            for (int64_t qs = per; qs < num_queries; qs += per) bounds.push_back(qs);
            bounds.push_back(num_queries);
        }
    } else if (num_queries > 0) {
        bounds.push_back(num_queries);
    }
    const int ranges = (int)bounds.size() - 1;  // 0 for an empty batch
    if (host_out) {
        const int rc = ensure_host_pipeline(g);
        if (rc) return rc;
    }

    // Walker ids continue across ranges (id_base = first query x walkers per
    // query), so the walks do not depend on how the batch is split.
    TRW_CUDA(cudaMemsetAsync(d_off, 0, sizeof(int64_t), st));
    const cudaStream_t rs[2] = {st, ranges > 1 ? g->aux_stream : st};
    if (rs[1] != st) {
        TRW_CUDA(cudaEventRecord(g->ev_fork, st));
        TRW_CUDA(cudaStreamWaitEvent(rs[1], g->ev_fork, 0));
    }
    int nr = 0;
    g->ppr_dirty = true;
    for (; nr < ranges; ++nr) {
        const int64_t qs = bounds[nr], nq = bounds[nr + 1] - qs;
        const cudaStream_t sr = rs[nr & 1];
        int32_t *tab = tables + (qs << (bits + 1));
        int32_t *dist = distinct + dist_ints * qs;
        int rc = run_walk(g, desc, d_src + qs, nq, nq * walkers_per_query, walkers_per_query, qs * walkers_per_query,
                          nullptr, 0, nullptr, nullptr, 0, false, d_steps + nr, engine, sr, tab, bits,
                          /*hold_lock=*/true);
        if (rc) {
            // earlier ranges are still queued on both streams: let them finish before returning
            if (rs[1] != st) cudaStreamSynchronize(rs[1]);
            cudaStreamSynchronize(st);
            return rc;
        }
        if (nr > 0 && rs[1] != st) TRW_CUDA(cudaStreamWaitEvent(sr, g->offsets_done[nr - 1], 0));
        TRW_CUDA(launch_ppr_offsets(tab, bits, dist, nq, d_off + qs, sr, cbits));
        if (host_out) TRW_CUDA(cudaEventRecord(g->offsets_done[nr], sr));
        TRW_CUDA(launch_ppr_emit(tab, bits, nq, d_off + qs, dist, d_v, d_c, capacity, g->error, sr, cbits));
        if (host_out) {
            TRW_CUDA(cudaMemcpyAsync(g->h_ends + nr, d_off + qs + nq, sizeof(int64_t), cudaMemcpyDeviceToHost, sr));
            TRW_CUDA(cudaEventRecord(g->range_done[nr], sr));
        }
    }
    if (rs[1] != st) {
        TRW_CUDA(cudaEventRecord(g->ev_join, rs[1]));
        TRW_CUDA(cudaStreamWaitEvent(st, g->ev_join, 0));
    }
    TRW_CUDA(cudaEventRecord(g->ppr_done, st));
    g->ppr_dirty = false;
    if (g->profile) {
        TRW_CUDA(cudaEventRecord(g->ev_post1, st));
        g->have_post = true;
    }
    if (steps) {
        uint64_t *sum = h_steps ? d_steps + kMaxRanges : steps;
        if (nr == 1) TRW_CUDA(cudaMemcpyAsync(sum, d_steps, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
        else TRW_CUDA(launch_sum_steps(d_steps, nr, sum, st));
        if (h_steps) TRW_CUDA(cudaMemcpyAsync(steps, sum, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    }
    int64_t total = 0;
    if (host_out) {
        int64_t prev = 0;
        for (int r = 0; r < nr; ++r) {
            TRW_CUDA(cudaEventSynchronize(g->range_done[r]));
            const int64_t end = g->h_ends[r];
            total = end;
            if (end <= capacity && end > prev) {
                const size_t n = sizeof(int32_t) * (size_t)(end - prev);
                if (h_v) TRW_CUDA(cudaMemcpyAsync(vertices + prev, d_v + prev, n, cudaMemcpyDeviceToHost, g->copy_stream));
                if (h_c) TRW_CUDA(cudaMemcpyAsync(counts + prev, d_c + prev, n, cudaMemcpyDeviceToHost, g->copy_stream));
            }
            prev = end;
        }
    }
    if (host_out || h_src || h_steps) {
        TRW_CUDA(cudaStreamSynchronize(st));
        if (h_off) TRW_CUDA(cudaMemcpyAsync(offsets, d_off, sizeof(int64_t) * (size_t)(num_queries + 1),
                                            cudaMemcpyDeviceToHost, g->copy_stream));
        if (host_out) TRW_CUDA(cudaStreamSynchronize(g->copy_stream));
        int err = 0;
        TRW_CUDA(cudaMemcpy(&err, g->error, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) {
            TRW_CUDA(cudaMemset(g->error, 0, sizeof(int)));
            if (err & kErrCapacity)
                return fail(TRW_ERR_CAPACITY, "sparse PPR output needs %lld entries, capacity is %lld",
                            (long long)total, (long long)capacity);
            return fail(TRW_ERR_DEVICE, "device error word %d (1 = rejection trial limit, 2 = invalid source vertex)",
                        err);
        }
    }
    return TRW_OK;
}

int trw_profile_enable(trw_graph *g, int32_t enable) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    for (cudaEvent_t *e : {&g->ev_walk0, &g->ev_walk1, &g->ev_post1})
        if (!*e) TRW_CUDA(cudaEventCreate(e));
    g->profile = enable != 0;
    g->have_post = false;
    return TRW_OK;
}

int trw_profile_read(trw_graph *g, float *walk_ms, float *post_ms) {
    if (!g || !g->profile) return fail(TRW_ERR_INVALID, "profiling is not enabled on this graph");
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    TRW_CUDA(cudaEventSynchronize(g->have_post ? g->ev_post1 : g->ev_walk1));
    float a = 0.f, b = 0.f;
    TRW_CUDA(cudaEventElapsedTime(&a, g->ev_walk0, g->ev_walk1));
    if (g->have_post) TRW_CUDA(cudaEventElapsedTime(&b, g->ev_walk1, g->ev_post1));
    if (walk_ms) *walk_ms = a;
    if (post_ms) *post_ms = b;
    return TRW_OK;
}

int trw_set_engine_shape(trw_graph *g, int32_t sampler, int32_t walkers_per_thread, int32_t ctas_per_sm) {
    if (!g || sampler < 0 || sampler > 4) return fail(TRW_ERR_INVALID, "bad arguments");
    if (walkers_per_thread != 0 && walkers_per_thread != 1 && walkers_per_thread != 2 && walkers_per_thread != 4 &&
        walkers_per_thread != 8 && walkers_per_thread != -1)
        return fail(TRW_ERR_INVALID, "walkers per thread must be 1, 2, 4 or 8 (0 automatic, -1 the plain form)");
    std::lock_guard<std::mutex> lock(g->mu);
    g->shape[sampler].ring = walkers_per_thread;  // 0 = automatic, -1 = the plain form
    g->shape[sampler].ctas_per_sm = ctas_per_sm > 0 ? ctas_per_sm : 0;
    return TRW_OK;
}

int trw_get_engine_shape(const trw_graph *g, int32_t sampler, int32_t *walkers_per_thread, int32_t *ctas_per_sm) {
    if (!g || sampler < 0 || sampler > 4) return fail(TRW_ERR_INVALID, "bad arguments");
    if (walkers_per_thread) *walkers_per_thread = g->shape[sampler].ring;
    if (ctas_per_sm) *ctas_per_sm = g->shape[sampler].ctas_per_sm;
    return TRW_OK;
}

int trw_device_error(trw_graph *g, int32_t *code) {
    if (!g || !code) return fail(TRW_ERR_INVALID, "null argument");
    TRW_CUDA(cudaSetDevice(g->device));
    TRW_CUDA(cudaDeviceSynchronize());
    int v = 0;
    TRW_CUDA(cudaMemcpy(&v, g->error, sizeof(int), cudaMemcpyDeviceToHost));
    TRW_CUDA(cudaMemset(g->error, 0, sizeof(int)));
    *code = v;
    return TRW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched walks of the serving loop (trw_batch.h).
// ---------------------------------------------------------------------------

int32_t trw::batch_ppr_bits(const trw_graph *g, int64_t walkers, double tp) {
    // as trw_ppr_batch_sparse: 2^bits >= 1.25 x the expected visits, <= 2 n
    const double visits = (double)walkers / tp;
    int32_t bits = 10;
    while (bits < 30 && (double)(1ll << bits) < 1.25 * visits) ++bits;
    while (bits > 10 && (1ll << (bits - 1)) >= 2ll * g->n) --bits;
    return bits;
}

int64_t trw::batch_ppr_distinct_ints(int32_t bits) { return ppr_distinct_ints(bits); }

int trw::batch_walk(trw_graph *g, std::vector<BatchItem> &items, cudaStream_t st, std::vector<int> &host_done) {
    if (!g) return fail(TRW_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lock(g->mu);
    TRW_CUDA(cudaSetDevice(g->device));
    host_done.clear();
    // plan every request; group the thread-engine ones by kernel
    struct Key {
        int sampler, update, wk;
        bool operator<(const Key &o) const {
            return sampler != o.sampler ? sampler < o.sampler : update != o.update ? update < o.update : wk < o.wk;
        }
    };
    std::vector<std::pair<Key, int>> shared;
    std::vector<int> alone;
    std::vector<Plan> plans(items.size());
    for (int i = 0; i < (int)items.size(); ++i) {
        BatchItem &it = items[(size_t)i];
        Plan &pl = plans[(size_t)i];
        int rc = make_plan(g, &it.desc, pl);
        if (rc) return rc;
        rc = prepare_plan(g, &it.desc, pl, st);
        if (rc) return rc;
        if (it.num_walkers <= 0) { host_done.push_back(i); continue; }
        if (pl.warp_family) alone.push_back(i);
        else shared.push_back({Key{pl.sampler, pl.update, pl.weight_kind}, i});
    }
    std::stable_sort(shared.begin(), shared.end(),
                     [](const std::pair<Key, int> &a, const std::pair<Key, int> &b) { return a.first < b.first; });
    for (size_t a = 0; a < shared.size();) {
        size_t b = a;
        while (b < shared.size() && !(shared[a].first < shared[b].first) && !(shared[b].first < shared[a].first)) ++b;
        const Key key = shared[a].first;
        const int k = (int)(b - a);
        // device request table: parameters, chunk prefix, PPR tables and
        // table sizes, walkers left, completion flags, queue head
        const size_t b_p = align_up(sizeof(WalkParams) * (size_t)k);
        const size_t b_c = align_up(sizeof(int64_t) * (size_t)(k + 1));
        const size_t b_t = align_up(sizeof(int32_t *) * (size_t)k);
        const size_t b_b = align_up(sizeof(int32_t) * (size_t)k);
        const size_t b_r = align_up(sizeof(int32_t) * (size_t)k);
        const size_t b_d = align_up(sizeof(int32_t *) * (size_t)k);
        const size_t bytes = b_p + b_c + b_t + b_b + b_r + b_d + sizeof(unsigned long long);
        std::vector<char> h(bytes, 0);
        WalkParams *hp = reinterpret_cast<WalkParams *>(h.data());
        int64_t *hc = reinterpret_cast<int64_t *>(h.data() + b_p);
        int32_t **ht = reinterpret_cast<int32_t **>(h.data() + b_p + b_c);
        int32_t *hb = reinterpret_cast<int32_t *>(h.data() + b_p + b_c + b_t);
        int32_t *hr = reinterpret_cast<int32_t *>(h.data() + b_p + b_c + b_t + b_b);
        volatile int32_t **hd = reinterpret_cast<volatile int32_t **>(h.data() + b_p + b_c + b_t + b_b + b_r);
        bool any_table = false;
        int64_t walkers = 0;
        hc[0] = 0;
        for (int j = 0; j < k; ++j) {
            const BatchItem &it = items[(size_t)shared[a + (size_t)j].second];
            const Plan &pl = plans[(size_t)shared[a + (size_t)j].second];
            WalkParams &p = hp[j];
            p.g = dev_view(g);
            if (pl.sampler == kLabelIndex) p.g.lab_fat = lab_fat_for(g, &it.desc);
            fill_app_params(p, &it.desc);
            p.static_unit = pl.table_kind == TRW_WEIGHTS_UNIT;
            p.sources = it.sources;
            p.num_walkers = it.num_walkers;
            p.per_query = it.per_query;
            p.id_base = it.id_base;
            p.paths = it.paths;
            p.path_cap = it.paths ? it.path_cap : 0;
            p.path_vec = it.paths && it.path_cap % 4 == 0 && reinterpret_cast<uintptr_t>(it.paths) % 16 == 0;
            p.lengths = it.lengths;
            p.steps = reinterpret_cast<unsigned long long *>(it.steps);
            p.error = g->error;
            hc[j + 1] = hc[j] + (it.num_walkers + kMultiChunk - 1) / kMultiChunk;
            ht[j] = it.table;
            hb[j] = it.table_bits;
            hr[j] = (int32_t)it.num_walkers;
            hd[j] = it.table ? nullptr : it.done;  // PPR requests finish after their post-processing
            any_table |= it.table != nullptr;
            walkers += it.num_walkers;
        }
        char *d = nullptr;
        TRW_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&d), bytes, st));
        // from pageable memory: the call returns once `h` has been staged
        TRW_CUDA(cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, st));
        MultiBatch mb;
        mb.reqs = reinterpret_cast<const WalkParams *>(d);
        mb.chunk_start = reinterpret_cast<const int64_t *>(d + b_p);
        mb.nreq = k;
        mb.tables = any_table ? reinterpret_cast<int32_t *const *>(d + b_p + b_c) : nullptr;
        mb.table_bits = reinterpret_cast<const int32_t *>(d + b_p + b_c + b_t);
        mb.remaining = reinterpret_cast<int32_t *>(d + b_p + b_c + b_t + b_b);
        mb.done = reinterpret_cast<volatile int32_t *const *>(d + b_p + b_c + b_t + b_b + b_r);
        mb.queue_head = reinterpret_cast<unsigned long long *>(d + b_p + b_c + b_t + b_b + b_r + b_d);
        mb.error = g->error;
        const cudaError_t le = launch_walk_multi(mb, walkers, hc[k], key.sampler, key.update, key.wk, g->num_sms, st);
        if (le != cudaSuccess) return fail(TRW_ERR_CUDA, "batched walk launch: %s", cudaGetErrorString(le));
        TRW_CUDA(cudaFreeAsync(d, st));
        for (int j = 0; j < k; ++j) {
            const int i = shared[a + (size_t)j].second;
            if (!items[(size_t)i].done || items[(size_t)i].table) host_done.push_back(i);
        }
        a = b;
    }
    for (int i : alone) {
        BatchItem &it = items[(size_t)i];
        const int rc = run_walk(g, &it.desc, it.sources, it.per_query > 0 ? it.num_walkers / it.per_query : it.num_walkers,
                                it.num_walkers, it.per_query, it.id_base, it.paths,
                                it.path_cap, it.lengths, nullptr, 0, false, it.steps, TRW_ENGINE_PERSISTENT, st,
                                nullptr, 0, /*hold_lock=*/true);
        if (rc) return rc;
        host_done.push_back(i);
    }
    // single-query PPR requests: their table into CSR
    for (BatchItem &it : items) {
        if (!it.table) continue;
        TRW_CUDA(cudaMemsetAsync(it.offsets, 0, sizeof(int64_t), st));
        TRW_CUDA(launch_ppr_offsets(it.table, it.table_bits, it.distinct, 1, it.offsets, st));
        TRW_CUDA(launch_ppr_emit(it.table, it.table_bits, 1, it.offsets, it.distinct, it.vertices, it.counts,
                                 it.capacity, g->error, st));
    }
    std::sort(host_done.begin(), host_done.end());
    return TRW_OK;
}

// ---------------------------------------------------------------------------
// Dynamic-alias walks that allocate nothing.
//
// Some callers cannot call cudaMalloc when they walk: code running inside a
// framework that owns all device memory through its own pool and forbids
// other allocators, latency-critical serving threads where a
// cudaMalloc/cudaFree would synchronise the whole device, and hosts with a
// device-memory budget fixed at start-up.  trw_walk allocates the per-warp
// alias tables of the dynamic-alias kernel on demand; this entry point runs
// the same kernel with those tables in the fixed array below instead.
//
// The array is a file-scope device variable: every GPU that loads this
// library holds kNoAllocScratchBytes of it until the process exits.  Its
// first 256 bytes hold the call's work-queue head and step counter (cleared
// by every call); the rest holds one raw + one table row of max_degree alias
// slots per warp.  Host code only ever sees a host-side stand-in for the
// symbol, so the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and cached.
// ---------------------------------------------------------------------------

static constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB per GPU
static constexpr size_t kNoAllocStateBytes = 256;          // queue head + step counter
static __device__ __align__(256) unsigned char trw_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_base[kNoAllocMaxDevices];

// Device address of trw_noalloc_scratch on `device` (which must be current).
int noalloc_scratch_base(int device, unsigned char **out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return fail(TRW_ERR_INVALID, "device %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[device]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, trw_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(TRW_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
        g_noalloc_base[device] = static_cast<unsigned char *>(ptr);
    }
    *out = g_noalloc_base[device];
    return TRW_OK;
}

}  // namespace

extern "C" int trw_walk_dynamic_alias_noalloc(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources,
                                              int64_t num_walkers, int64_t id_base, int32_t *paths,
                                              int32_t path_cap, int32_t *lengths, int32_t *counts,
                                              uint64_t *steps, trw_stream_t stream) {
    if (!g || !desc) return fail(TRW_ERR_INVALID, "null graph or descriptor");
    if (desc->mode != TRW_MODE_DYNAMIC || desc->sampler != TRW_SAMPLER_ALIAS)
        return fail(TRW_ERR_UNSUPPORTED, "the no-alloc entry point runs dynamic-mode alias sampling only");
    if (num_walkers < 0 || (num_walkers > 0 && !sources)) return fail(TRW_ERR_INVALID, "bad walker arguments");
    if (paths && path_cap <= 0) return fail(TRW_ERR_INVALID, "path_cap must be > 0 when paths are requested");
    const void *ptrs[] = {sources, paths, lengths, counts, steps};
    for (const void *q : ptrs)
        if (q && !is_device_ptr(q))
            return fail(TRW_ERR_INVALID, "the no-alloc entry point takes device pointers only (staging would allocate)");
    // The graph's lookup structures (edge set, label index), launch shapes
    // and profiling events are written by other calls under this lock; hold
    // it from the plan through the launch, as trw_walk does.  A lock
    // allocates nothing.
    std::lock_guard<std::mutex> lock(g->mu);
    Plan pl;
    int rc = make_plan(g, desc, pl);
    if (rc) return rc;
    const int64_t stride = 2 * (int64_t)std::max(1, g->max_degree);
    const int64_t table_bytes = (int64_t)(kNoAllocScratchBytes - kNoAllocStateBytes);
    int64_t warps = table_bytes / ((int64_t)sizeof(AliasSlot) * stride) / 8 * 8;
    if (warps < 8)
        return fail(TRW_ERR_CAPACITY, "max degree %d needs %lld bytes of alias scratch for one CTA; the no-alloc scratch "
                    "holds %lld bytes (max degree <= %lld)", g->max_degree,
                    (long long)(8 * stride * (int64_t)sizeof(AliasSlot)), (long long)table_bytes,
                    (long long)(table_bytes / (8 * 2 * (int64_t)sizeof(AliasSlot))));
    TRW_CUDA(cudaSetDevice(g->device));
    unsigned char *base = nullptr;
    rc = noalloc_scratch_base(g->device, &base);
    if (rc) return rc;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long *state = reinterpret_cast<unsigned long long *>(base);
    TRW_CUDA(cudaMemsetAsync(state, 0, 2 * sizeof(unsigned long long), st));

    WalkParams p;
    std::memset(&p, 0, sizeof p);
    p.g = dev_view(g);
    fill_app_params(p, desc);
    p.sources = sources;
    p.num_walkers = num_walkers;
    p.id_base = id_base;
    p.paths = paths;
    p.path_cap = paths ? path_cap : 0;
    p.lengths = lengths;
    p.counts = counts;
    p.queue_head = state;
    p.steps = state + 1;
    p.error = g->error;
    p.alias_scratch = reinterpret_cast<AliasSlot *>(base + kNoAllocStateBytes);
    p.alias_scratch_stride = stride;

    LaunchShape shape = g->shape[kAlias];
    shape.engine = kEnginePersistent;
    shape.num_sms = g->num_sms;
    shape.max_warps = std::min(warps, warp_engine_warps(p, shape));
    if (g->profile) {  // event records allocate nothing
        TRW_CUDA(cudaEventRecord(g->ev_walk0, st));
        g->have_post = false;
    }
    const cudaError_t le = launch_walk_warp(p, kAlias, pl.update, pl.weight_kind, shape, st);
    if (le != cudaSuccess) return fail(TRW_ERR_CUDA, "walk launch: %s", cudaGetErrorString(le));
    if (g->profile) TRW_CUDA(cudaEventRecord(g->ev_walk1, st));
    if (steps) TRW_CUDA(cudaMemcpyAsync(steps, state + 1, sizeof(uint64_t), cudaMemcpyDeviceToDevice, st));
    return TRW_OK;
}
