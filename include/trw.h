/*
 * trw.h -- C ABI of libtrw_gpu.so, the GB300 random-walk engine.
 *
 * Drop-in boundary for ThunderRW's walk path (Gather-Move-Update,
 * random_walk/creeper.h).  The reference exposes header-only C++ templates
 * (compute<F>(Graph&, std::vector<WalkerMeta>&, F), creeper.h:689) with
 * per-app functors and process globals (g_para, types.h:109); this ABI carries
 * the same information as plain values and pointers so any host language can
 * bind it.  Every function returns TRW_OK (0) or a negative trw_status and
 * never aborts the process; trw_last_error() describes the last failure on
 * the calling thread.
 *
 * Pointers passed for walk inputs and outputs may be host or device memory:
 * the library inspects each pointer, stages host buffers through HBM and
 * copies host outputs back before returning (such calls synchronise the
 * stream).  With device pointers the call only enqueues work on `stream`.
 *
 * Randomness: every walker draws from Philox4x32-10 with
 *   key = (seed lo, seed hi), counter = (block, step, walker lo, walker hi),
 * where step is the walker's length before the move (1 for the first move),
 * draw d of one move uses block d/4 and word d%4, and the PPR termination
 * draw uses block TRW_TERM_BLOCK with step = length after the move.  Results
 * therefore do not depend on scheduling, engine choice or batching.
 */
#ifndef TRW_H
#define TRW_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct trw_graph trw_graph;
typedef struct CUstream_st *trw_stream_t; /* a cudaStream_t; NULL = legacy default stream */

#define TRW_TERM_BLOCK 0x80000000u

enum trw_status {
    TRW_OK = 0,
    TRW_ERR_INVALID = -1,      /* bad argument */
    TRW_ERR_CUDA = -2,         /* CUDA runtime error (message in trw_last_error) */
    TRW_ERR_UNSUPPORTED = -3,  /* app / mode / sampler combination not supported */
    TRW_ERR_NO_TABLES = -4,    /* static sampler used before trw_tables_build */
    TRW_ERR_GRAPH = -5,        /* graph failed validation */
    TRW_ERR_DEVICE = -6,       /* a kernel raised its device error word */
    TRW_ERR_CAPACITY = -7,     /* size above a stated maximum */
    TRW_ERR_BUSY = -8          /* serving queue full */
};

/* App hooks (random_walk/apps/<app>.cpp).  DeepWalk and GenericWalk share hooks:
 * weight = edge weight, update = (length == l), max_weight = 5.0. */
enum trw_app {
    TRW_APP_DEEPWALK = 0,   /* deepwalk.cpp:9-30 */
    TRW_APP_PPR = 1,        /* ppr.cpp:10-34: weight 1, update real1 <= tp */
    TRW_APP_NODE2VEC = 2,   /* node2vec.cpp:9-47: weight {1/p, 1, 1/q} */
    TRW_APP_METAPATH = 3,   /* metapath.cpp:9-39: weight [label == schema[(len-1)%S]] */
    TRW_APP_GENERICWALK = 4 /* genericwalk.cpp:9-30 */
};

/* ExecutionMode (types.h:41-45) and SamplingMethod (types.h:53-59). */
enum trw_mode { TRW_MODE_UNIFORM = 0, TRW_MODE_STATIC = 1, TRW_MODE_DYNAMIC = 2 };
enum trw_sampler {
    TRW_SAMPLER_UNIFORM = 0,
    TRW_SAMPLER_ITS = 1,
    TRW_SAMPLER_ALIAS = 2,
    TRW_SAMPLER_REJECTION = 3,
    TRW_SAMPLER_MAXWEIGHT_REJECTION = 4
};

/* Static-table weights: what static_gather (creeper.h:24-99) produces for
 * the app: edge weights (DeepWalk, GenericWalk) or 1.0 (PPR). */
enum trw_weight_kind { TRW_WEIGHTS_EDGE = 0, TRW_WEIGHTS_UNIT = 1 };

/* Engine: the persistent batched engine (warps keep several walkers in
 * flight and refill them from a device work queue) or the plain form (one
 * thread per walker, one launch per call, no refill). */
enum trw_engine { TRW_ENGINE_PERSISTENT = 0, TRW_ENGINE_PLAIN = 1 };

/* AliasSlot (config/type_config.h:22-26), byte-identical layout. */
typedef struct {
    double prob;
    int32_t first;
    int32_t second;
} trw_alias_slot;

#define TRW_MAX_SCHEMA 64

/* The per-run parameters the reference takes from g_para (types.h:72-77,109)
 * and from the app functor's constructor arguments. */
typedef struct {
    int32_t app;          /* trw_app */
    int32_t mode;         /* trw_mode (g_para.execution_) */
    int32_t sampler;      /* trw_sampler (g_para.sample_) */
    int32_t length;       /* l_: walk length of the fixed-length apps */
    double p;             /* Node2Vec return parameter; return edges weigh 1/p */
    double q;             /* Node2Vec in-out parameter; other edges weigh 1/q */
    double tp;            /* PPR termination probability */
    const int32_t *schema;/* MetaPath schema (host memory), <= TRW_MAX_SCHEMA */
    int32_t schema_len;
    uint64_t seed;        /* Philox key */
} trw_walk_desc;

/* ---- graph ------------------------------------------------------------ */

#define TRW_GRAPH_CHECK_SORTED 1u  /* also verify sorted neighbour lists (graph.cpp:764-776) */

/* Replaces Graph::load_csr's in-memory result (util/graph/graph.cpp:45-101;
 * CSR arrays graph.h:51-65, offset_pair_ graph.cpp:86-91).  Copies the CSR
 * (row_ptr n+1 int64, adj e int32, optional weight e double, optional label
 * e int32) into library-owned HBM; the caller keeps its arrays.  Validates
 * row_ptr monotonicity, adjacency range and e < 2^31. */
int trw_graph_create(const int64_t *row_ptr, const int32_t *adj, const double *weight,
                     const int32_t *label, int32_t n, int64_t e, uint32_t flags,
                     trw_graph **out);

/* Replaces Graph::~Graph (graph.h:118-145). */
int trw_graph_destroy(trw_graph *g);

/* num_vertices / num_edges / max_degree (graph.h:152-166). */
int trw_graph_info(const trw_graph *g, int32_t *n, int64_t *e, int32_t *max_degree);

/* Waits until all work the library enqueued for this graph, on any stream,
 * has finished (the reference's compute and static_initialization return
 * only when done; asynchronous callers use this as the join point). */
int trw_graph_synchronize(trw_graph *g);

/* Which lookup structures the graph's walks use (no counterpart in the
 * reference; each replaces a per-step search with a lookup and is built by
 * the first walk that needs it): the Node2Vec edge set (replacing
 * Graph::is_neighbor's binary search, graph.h:180-199) and the MetaPath
 * label index (replacing dynamic ITS's scan of the label row,
 * inverse_transformation_sampling.h:288-313).  Each state: 0 = not built
 * yet, 1 = built, -1 = not applicable (MetaPath labels outside [0, 64)) or
 * no room on the device; the walks then keep the searches.  Results are the
 * same either way. */
int trw_graph_indexes(const trw_graph *g, int32_t *edge_set_state, int32_t *label_index_state);

/* The layouts the walks read (no counterpart in the reference; results are
 * the same with either).  fat_adjacency_state, for uniform and max-weight
 * rejection walks: 1 = 16-byte adjacency entries that carry each neighbour's
 * offset pair (built by the first such walk when the offset pairs, 8 bytes
 * per vertex, exceed half the device's L2; a move then reads one entry
 * instead of the pair and then the entry), 0 = not decided yet, -1 = the
 * plain adjacency (small graph or no room).  fat_label_index_state, for
 * MetaPath walks on the label index whose schema names each label at most
 * once: 1 = 16-byte label-index entries that carry the next step's block of
 * positions, built by trw_walk for the last such schema (when the label
 * offsets, 4 (K + 1) bytes per vertex, exceed half the L2), 0 / -1 as
 * above.  The environment variable TRW_FAT_ADJACENCY=1 / 0, read when a
 * decision is made, forces both one way. */
int trw_graph_layout(const trw_graph *g, int32_t *fat_adjacency_state, int32_t *fat_label_index_state);

/* Builds those lookup structures now instead of in the first walk that needs
 * them, e.g. before a serving loop starts so that no request pays for a
 * build (the reference builds everything it needs before compute() starts
 * its timer, creeper.h:700-766).  Nonzero flags select the structures; one
 * already built, not applicable or without room is left as it is (read the
 * states with trw_graph_indexes).  edge_set also decides and builds the
 * adjacency entries with row pairs (trw_graph_layout).  Synchronises the
 * stream. */
int trw_graph_build_indexes(trw_graph *g, int32_t edge_set, int32_t label_index, trw_stream_t stream);

/* ---- static tables ---------------------------------------------------- */

/* Replaces static_initialization (creeper.h:102-175) and the offline
 * builders alias_preprocess.cpp:30-73, its_preprocess.cpp:21-34 and
 * rejection_preprocess.cpp:24-27: builds the alias table, the ITS prefix
 * sums or the rejection per-vertex maxima in HBM with device kernels,
 * bit-identical to the reference's sequential double arithmetic. */
int trw_tables_build(trw_graph *g, int32_t sampler, int32_t weight_kind, trw_stream_t stream);

/* Copies a built table to `out` (host or device): alias -> e trw_alias_slot
 * (edge_weight_alias_table_, graph.h:77), ITS -> e doubles
 * (edge_weight_prefix_sum_, graph.h:70), rejection -> n doubles
 * (edge_weight_rejection_max_, graph.h:83). */
int trw_tables_download(const trw_graph *g, int32_t sampler, void *out, size_t out_bytes);

/* Installs a precomputed table (host or device memory, the layout
 * trw_tables_download produces and the reference's preprocessors write:
 * b_edge_weight_alias_table.bin, b_edge_weight_prefix_sum.bin,
 * b_edge_weight_max.bin) as the graph's table for `sampler` built with
 * `weight_kind` weights, so that static walks with those weights use it
 * without building one.  Replaces the loading of those files by
 * Graph::load_csr (graph.cpp:78-94) under -ep / -al / -rj
 * (creeper_main.h:44-55).  `bytes` must be the table's size (alias: e x 16,
 * ITS: e x 8, rejection: n x 8).  A table the walks may still be reading is
 * replaced only after the device has finished them.  The reference's
 * compute() rebuilds its tables from the edge weights even when the files
 * were loaded (creeper.h:107-108); a table built by the reference's
 * preprocessors or by trw_tables_build is bit-identical to that rebuild. */
int trw_tables_upload(trw_graph *g, int32_t sampler, int32_t weight_kind, const void *table, size_t bytes,
                      trw_stream_t stream);

/* ---- walks ------------------------------------------------------------ */

/* Replaces compute<F>(graph, walkers, f) (creeper.h:689-831) for the five
 * reference apps, every mode x sampler pair of types.h:41-59.
 *   sources[i]      start vertex of walker i (WalkerMeta::source_, walker.h:9-15)
 *   id_base         Philox walker id of walker 0 (walker i uses id_base + i)
 *   paths           num_walkers x path_cap int32, walker-major, or NULL; entry
 *                   k < length holds the k-th vertex of the walk (seq_[k],
 *                   creeper.h:310-317), later entries are -1
 *   lengths         num_walkers int32 final length_ values, or NULL
 *   counts          n int32 visit counters, or NULL: every move adds 1 to
 *                   counts[new vertex] (so sum(counts) = steps); counts are
 *                   added to, not overwritten
 *   steps           receives the number of moves (creeper.h:305), or NULL
 * Walkers at a vertex without neighbours stop (the reference divides by zero
 * there).  With host paths / lengths and at least four walkers per lane of
 * the GPU (SMs x 2048), the walkers run as up to 16 ranges whose outputs are
 * copied back while the next range walks; the results are those of one
 * launch. */
int trw_walk(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_walkers,
             int64_t id_base, int32_t *paths, int32_t path_cap, int32_t *lengths, int32_t *counts,
             uint64_t *steps, int32_t engine, trw_stream_t stream);

/* Batched PPR: num_queries queries of walkers_per_query walkers each, all
 * in one launch.  Walker j of query q starts at sources[q] and has Philox id
 * q * walkers_per_query + j.  counts is num_queries x n int32 (query-major);
 * each move adds 1 to counts[q][new vertex].  With TRW_PPR_ZERO_COUNTS the
 * library zeroes counts first; otherwise counts are added to.  The reference
 * runs PPR as one compute() per source with no visit counter (ppr.cpp:37-84,
 * walker_generator.cpp:42-63); this entry point replaces a loop of those. */
#define TRW_PPR_ZERO_COUNTS 1u
int trw_ppr_batch(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_queries,
                  int64_t walkers_per_query, int32_t *counts, uint64_t *steps, uint32_t flags,
                  int32_t engine, trw_stream_t stream);

/* Batched PPR with sparse output: the same walks as trw_ppr_batch, but the
 * visit counts come back as per-query (vertex, count) lists instead of a
 * dense num_queries x n array.  Query q's entries are
 * vertices[offsets[q] .. offsets[q+1]) with their counts in counts[...];
 * only vertices with a non-zero count appear, in a canonical order that
 * depends on the counts alone (not on scheduling).  offsets has
 * num_queries + 1 entries; vertices and counts hold `capacity` entries.  If
 * the batch needs more than `capacity` entries, offsets is still written
 * (offsets[num_queries] is the size needed), at most the queries whose
 * entries end within `capacity` are written (with host outputs, only whole
 * query ranges that do), and the call reports TRW_ERR_CAPACITY (synchronous
 * calls) or device error 4: grow the buffers to offsets[num_queries] and
 * call again.  With host outputs a large batch
 * runs as several ranges of queries whose entries are copied back while the
 * next range walks; the output is that of one range. */
int trw_ppr_batch_sparse(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources, int64_t num_queries,
                         int64_t walkers_per_query, int64_t *offsets, int32_t *vertices, int32_t *counts,
                         int64_t capacity, uint64_t *steps, int32_t engine, trw_stream_t stream);

/* Launch shape of the persistent engine for this graph and sampler: walkers
 * per thread (ring depth 1, 2, 4 or 8) and CTAs per SM.  0 = automatic (ring
 * 1 for sparse PPR tables or fewer than 4 x SMs x 2048 walkers, else 4; as
 * many CTAs as fit).  walkers_per_thread = -1 makes persistent-engine calls
 * with this sampler run the plain form instead (one thread per walker, no
 * refill: the form some fixed-length walks run fastest in; the warp-family
 * kernels keep their own).  thunderrw_gb300/autotune.py measures and sets
 * them.  Walks are the same under every shape. */
int trw_set_engine_shape(trw_graph *g, int32_t sampler, int32_t walkers_per_thread, int32_t ctas_per_sm);
int trw_get_engine_shape(const trw_graph *g, int32_t sampler, int32_t *walkers_per_thread,
                         int32_t *ctas_per_sm);

/* Dynamic-mode alias walks (TRW_MODE_DYNAMIC + TRW_SAMPLER_ALIAS, any app)
 * that allocate nothing: no cudaMalloc, cudaFree or allocating library call.
 * No counterpart in the reference; it is for callers that cannot allocate
 * device memory while they walk (a framework that owns every device byte
 * through its own pool, serving threads where an allocation would
 * synchronise the device, hosts with a device-memory budget fixed at
 * start-up).  trw_walk allocates the kernel's per-warp alias tables on
 * demand; this entry point keeps them in a fixed 16 MiB device array that
 * every GPU loading the library holds until exit, so graphs whose maximum
 * degree exceeds 65535 are rejected with TRW_ERR_CAPACITY.  Arguments and
 * results are those of trw_walk, except that every non-NULL pointer must be
 * device memory (staging host buffers would allocate; host pointers give
 * TRW_ERR_INVALID) and the call is always asynchronous on `stream`.  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls on a device share the array: the
 * call clears the work-queue head and step counter it keeps there, and
 * calls that overlap on the GPU race on it, so serialise them (one stream,
 * or events).  The call holds the graph's lock from its checks through the
 * launch, like trw_walk, and is timed by trw_profile_read like any walk. */
int trw_walk_dynamic_alias_noalloc(trw_graph *g, const trw_walk_desc *desc, const int32_t *sources,
                                   int64_t num_walkers, int64_t id_base, int32_t *paths, int32_t path_cap,
                                   int32_t *lengths, int32_t *counts, uint64_t *steps, trw_stream_t stream);

/* Per-call timing (the GPU counterpart of the reference's walking-time
 * log, creeper.h:411-415,800-803).  While enabled, every walk call records
 * CUDA events on its stream around its walk-kernel launch and, for
 * trw_ppr_batch_sparse, after its post-processing launches; trw_profile_read
 * waits for the last call and returns the two durations in ms. */
int trw_profile_enable(trw_graph *g, int32_t enable);
int trw_profile_read(trw_graph *g, float *walk_ms, float *post_ms);

/* ---- serving ---------------------------------------------------------- */

/* A request loop over a resident graph (no counterpart in the reference,
 * which runs one compute() per process).  Requests of any app and size are
 * admitted in arrival order: whenever one of `max_inflight` streams is free,
 * every queued request whose device memory still fits `hbm_budget_bytes` (0 =
 * 80 % of the free HBM at start) joins one batch on that stream, and the
 * walkers of the batch's requests that use the same kernel run in one shared
 * persistent launch (one work queue over all of them).  Batches on different
 * streams overlap on the device.  A request completes when its last walker
 * does (single-query PPR requests: when their post-processing does).
 * Results stay in HBM until trw_server_release. */
typedef struct trw_server trw_server;

typedef struct {
    trw_walk_desc desc;
    const int32_t *sources;     /* host memory, copied at submit: num_walkers (walks) or num_queries (PPR) */
    int64_t num_walkers;        /* walks: walker count */
    int64_t id_base;            /* walks: Philox id of walker 0 */
    int32_t path_cap;           /* walks: path entries per walker, 0 = lengths only */
    int64_t num_queries;        /* sparse PPR batch: number of queries */
    int64_t walkers_per_query;  /* > 0: the request is trw_ppr_batch_sparse */
} trw_request;

typedef struct {
    int32_t state;       /* 0 queued, 1 running, 2 done, 3 failed */
    double latency_ms;   /* submit -> results complete in HBM */
    double queue_ms;     /* submit -> launch */
    uint64_t steps;
    int64_t entries;     /* sparse PPR: (vertex, count) entries */
} trw_request_status;

typedef struct {
    uint64_t submitted, completed, failed, steps;
    int64_t queued, running;
    size_t hbm_in_use;
    double p50_ms, p99_ms, max_ms, elapsed_s;
    uint64_t batches;    /* batches launched (each: one persistent launch per kernel of its requests) */
} trw_serving_stats;

int trw_server_start(trw_graph *g, size_t hbm_budget_bytes, int32_t max_inflight, trw_server **out);
/* TRW_ERR_BUSY when the queue is full, TRW_ERR_CAPACITY when the request
 * alone exceeds the budget. */
int trw_server_submit(trw_server *s, const trw_request *req, uint64_t *ticket);
/* Waits up to timeout_ms (< 0: forever) for the request to finish. */
int trw_server_wait(trw_server *s, uint64_t ticket, int32_t timeout_ms, trw_request_status *status);
/* Copies a finished request's outputs to host buffers (walks: paths,
 * lengths; PPR: offsets, and vertices/counts of `capacity` entries). */
int trw_server_result(trw_server *s, uint64_t ticket, int32_t *paths, int32_t *lengths, int64_t *offsets,
                      int32_t *vertices, int32_t *counts, int64_t capacity);
int trw_server_release(trw_server *s, uint64_t ticket);
int trw_server_stats(trw_server *s, trw_serving_stats *out);
/* Finishes the queued and running requests, then frees everything. */
int trw_server_stop(trw_server *s);

/* ---- errors ----------------------------------------------------------- */

/* Message of the last failure on the calling thread ("" if none). */
const char *trw_last_error(void);

/* Reads and clears the graph's device error word (1 = a rejection sampler
 * exceeded its trial limit, 2 = invalid vertex met in a walk). */
int trw_device_error(trw_graph *g, int32_t *code);

/* Library version, e.g. 1000 for 1.0.0. */
int32_t trw_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TRW_H */
