// trw_batch.h -- the serving loop's batched walk (internal; not part of the
// public ABI in include/trw.h).
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "trw.h"

namespace trw {

// One request of a batch; every pointer is device memory owned by the caller.
struct BatchItem {
    trw_walk_desc desc;        // desc.schema points to host memory
    const int32_t *sources;
    int64_t num_walkers;
    int64_t per_query;         // > 0: walker i starts at sources[i / per_query]
    int64_t id_base;
    int32_t *paths;            // walks: [num_walkers][path_cap] or null
    int32_t path_cap;
    int32_t *lengths;          // walks: [num_walkers] or null
    uint64_t *steps;           // zeroed by the caller
    // single-query PPR with sparse output: a zeroed table of 2^table_bits
    // keys followed by 2^table_bits counts, the CSR outputs and the
    // post-processing scratch (ppr_distinct_ints(table_bits) ints)
    int32_t *table;
    int32_t table_bits;
    int64_t *offsets;
    int32_t *vertices, *counts;
    int64_t capacity;
    int32_t *distinct;
    volatile int32_t *done;    // host-mapped completion flag (walks in a shared launch), or null
};

// Table size of a single-query PPR request (as trw_ppr_batch_sparse sizes it).
int32_t batch_ppr_bits(const trw_graph *g, int64_t walkers, double tp);
int64_t batch_ppr_distinct_ints(int32_t bits);

// Runs a batch of requests on `st`: the thread-engine requests as one
// persistent launch per (sampler, update rule, weight kind), the others as
// launches of their own; PPR requests are post-processed into their CSR
// outputs after their launch.  Walk requests of a shared launch raise their
// `done` flag from the device when their last walker finishes; the indexes
// of the other requests (which complete with the stream) go to `host_done`.
// The batch's own device tables are allocated and freed in stream order on
// `st`.
int batch_walk(trw_graph *g, std::vector<BatchItem> &items, cudaStream_t st, std::vector<int> &host_done);

}  // namespace trw
