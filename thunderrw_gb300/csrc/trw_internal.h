// trw_internal.h -- host-side declarations shared by the library's
// translation units (not part of the public ABI; see include/trw.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "trw_device.cuh"

namespace trw {

constexpr int kThreadBlock = 256;
constexpr int kEnginePersistent = 0;
constexpr int kEnginePlain = 1;

struct LaunchShape {
    int engine = kEnginePersistent;
    int ring = 0;         // walkers in flight per lane (thread family); 0 = automatic
    int ctas_per_sm = 0;  // 0 = as many as fit
    int num_sms = 1;
    int64_t max_warps = 0;  // dynamic alias: warps with a scratch table
};

cudaError_t launch_walk_thread(const WalkParams &p, int sampler, int update, int weight_kind,
                               const LaunchShape &shape, cudaStream_t st);
cudaError_t launch_walk_warp(const WalkParams &p, int sampler, int update, int weight_kind,
                             const LaunchShape &shape, cudaStream_t st);
// number of per-warp dynamic-alias scratch tables the warp engine will use
int64_t warp_engine_warps(const WalkParams &p, const LaunchShape &shape);

// Many requests in one persistent launch (the serving loop's batches): the
// walkers of all requests share one queue of chunks of kMultiChunk walkers,
// request r owning chunks [chunk_start[r], chunk_start[r + 1]).  reqs[r]
// holds request r's parameters with no visit-count outputs; a request with
// tables[r] != null (single-query PPR) records its visits in that
// 2^table_bits[r]-slot table (the layout of WalkParams::table).  remaining[r]
// starts at the request's walker count; the lane that finishes its last
// walker writes 1 to *done[r] (host-mapped memory) if done[r] is set.  All
// requests share the sampler, update rule and weight kind of the launch.
constexpr int kMultiChunk = 64;
struct MultiBatch {
    const WalkParams *reqs;
    const int64_t *chunk_start;
    int32_t nreq;
    int32_t *const *tables;
    const int32_t *table_bits;
    int32_t *remaining;
    volatile int32_t *const *done;
    unsigned long long *queue_head;
    int *error;
};
cudaError_t launch_walk_multi(const MultiBatch &mb, int64_t total_walkers, int64_t total_chunks, int sampler,
                              int update, int weight_kind, int num_sms, cudaStream_t st);

// Sparse PPR post-processing takes a table in chunks of at most
// 2^chunk_bits slots, one CTA each (10 <= chunk_bits <= 16); the same
// chunk_bits must reach ppr_distinct_ints, launch_ppr_offsets and
// launch_ppr_emit of one batch.  A chunked table (more than one chunk) is
// zeroed by a memset after its emit instead of by the emit's CTA.
constexpr int32_t kPprChunkBits = 16;
// offsets[0] must hold the entries before this range of queries (0 for the first)
cudaError_t launch_ppr_offsets(const int32_t *tables, int32_t bits, int32_t *distinct, int64_t nq, int64_t *offsets,
                               cudaStream_t st, int32_t chunk_bits = kPprChunkBits);
// `distinct` holds nq totals followed by ppr_distinct_ints(bits) - 1 segment
// prefixes per query (ppr_distinct_ints(bits) ints per query in all)
int64_t ppr_distinct_ints(int32_t bits, int32_t chunk_bits = kPprChunkBits);
cudaError_t launch_ppr_emit(int32_t *tables, int32_t bits, int64_t nq, const int64_t *offsets,
                            const int32_t *distinct, int32_t *vout, int32_t *cout, int64_t capacity, int *error,
                            cudaStream_t st, int32_t chunk_bits = kPprChunkBits);
// *out = parts[0] + ... + parts[n-1], on the device
cudaError_t launch_sum_steps(const uint64_t *parts, int n, uint64_t *out, cudaStream_t st);

// (degree, vertex) of the rows the warp builders take, appended in any order
cudaError_t launch_collect_long_rows(const DevGraph &g, int2 *list, int *count, cudaStream_t st);
// long_rows: the vertices of rows longer than 32 entries (longest first), one warp each
cudaError_t launch_build_alias(const DevGraph &g, int unit, AliasSlot *out, const int32_t *long_rows,
                               int32_t n_long, cudaStream_t st);
// *bad |= 1 if some edge weight is negative or NaN or a non-empty row has no positive weight
cudaError_t launch_positive_rows(const DevGraph &g, int *bad, cudaStream_t st);
// lo_hi[0] / lo_hi[1] (preset to INT_MAX / INT_MIN) become the smallest and
// largest edge label
cudaError_t launch_label_range(const int32_t *label, int64_t e, int *lo_hi, cudaStream_t st);
// MetaPath's label index for labels in [0, K): off[n * (K + 1)], nbr[e]
cudaError_t launch_build_label_index(const DevGraph &g, int32_t K, int32_t *off, int32_t *nbr, cudaStream_t st);
// Node2Vec's edge set: `set` (2^bits slots) must hold kEdgeEmpty everywhere;
// *symmetric must hold 1 and is cleared if some edge's reverse is missing.
cudaError_t launch_build_edge_set(const DevGraph &g, unsigned long long *set, int32_t bits, int *symmetric,
                                  cudaStream_t st);
// DevGraph::lab_fat for every label-index entry (g.lab_off / g.lab_nbr
// read): label[l] = the label a step wants after one along a label-l edge
struct LabelNext {
    int32_t label[kMaxIndexedLabels];
};
cudaError_t launch_build_lab_fat(const DevGraph &g, const LabelNext &next, int4 *fat, cudaStream_t st);
// DevGraph::fat for every edge (g.rows and g.adj are read)
cudaError_t launch_build_fat(const DevGraph &g, int4 *fat, cudaStream_t st);
cudaError_t launch_build_prefix(const DevGraph &g, int unit, double *out, const int32_t *long_rows,
                                int32_t n_long, cudaStream_t st);
cudaError_t launch_build_max(const DevGraph &g, int unit, double *out, cudaStream_t st);
cudaError_t launch_validate_graph(const int64_t *row, const int32_t *adj, int32_t n, int64_t e, int check_sorted,
                                  int2 *rows_out, int *bad, int *max_degree, cudaStream_t st);

}  // namespace trw
