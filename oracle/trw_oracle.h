/*
 * trw_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of ThunderRW's Gather-Move-Update walk path, the oracle
 * the GPU engine is tested against.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  The product path
 * (libtrw_gpu.so) never links or calls anything here.
 *
 * Every function restates the reference's algorithm (file:line cited beside
 * it, paths relative to the ThunderRW source tree).  Uniforms come from the
 * counter-based Philox4x32-10 contract shared with the GPU kernels:
 *
 *   key     = { (u32)seed, (u32)(seed >> 32) }
 *   counter = { block, (u32)step, (u32)walker, (u32)(walker >> 32) }
 *   step    = the walker's length_ at draw time (1 for the first move)
 *   draw d of one (walker, step) move uses block d/4, output word d%4
 *   the PPR termination draw (ppr.cpp:27-29) uses block TRW_TERM_BLOCK,
 *   word 0, with step = length_ after the move.
 *
 * u32 -> double conversions are SFMT's (SFMT.h:193-228):
 *   real1(v) = v * (1.0/4294967295.0),  real2(v) = v * (1.0/4294967296.0).
 */
#ifndef TRW_ORACLE_H
#define TRW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_TERM_BLOCK 0x80000000u

/* Mirrors AliasSlot (config/type_config.h:22-26): 16 bytes. */
typedef struct {
    double prob;
    int32_t first;
    int32_t second;
} oracle_alias_slot;

typedef struct {
    int32_t n;                 /* vertices */
    int64_t e;                 /* directed CSR entries */
    const int64_t *row;        /* n+1 offsets (graph.h:51) */
    const int32_t *adj;        /* e neighbour ids, sorted per row */
    const double *weight;      /* e edge weights or NULL (graph.h:65) */
    const int32_t *label;      /* e edge labels or NULL (graph.h:64) */
    const oracle_alias_slot *alias; /* static alias table (graph.h:77) */
    const double *prefix;      /* static ITS prefix sums (graph.h:70) */
    const double *rej_weight;  /* static rejection weights (graph.h:82) */
    const double *rej_max;     /* static rejection per-vertex max (graph.h:83) */
} oracle_graph;

/* Numbering follows random_walk/types.h:41-59 for mode and sampler. */
typedef struct {
    int32_t app;          /* 0 DeepWalk, 1 PPR, 2 Node2Vec, 3 MetaPath, 4 GenericWalk */
    int32_t mode;         /* 0 Uniform, 1 Static, 2 Dynamic */
    int32_t sampler;      /* 0 Uniform, 1 ITS, 2 Alias, 3 Rejection, 4 MaxWeightRejection */
    int32_t length;       /* walk length l_ of the fixed-length apps */
    double p;             /* Node2Vec return parameter (weight 1/p) */
    double q;             /* Node2Vec in-out parameter (weight 1/q) */
    double tp;            /* PPR termination probability */
    const int32_t *schema;/* MetaPath schema */
    int32_t schema_len;
    uint64_t seed;
} oracle_walk_desc;

/* Philox4x32-10 (Salmon et al., SC'11). */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* The u32 draw #d of (seed, walker, step), and the PPR termination draw. */
uint32_t oracle_draw_u32(uint64_t seed, uint64_t walker, uint32_t step, uint32_t d);

/* Static table builders.  weight_kind: 0 edge weights, 1 unit weights (the
 * static_gather of the app's weight hook, creeper.h:24-99). */
int oracle_build_alias(const oracle_graph *g, int weight_kind, oracle_alias_slot *out);
int oracle_build_prefix(const oracle_graph *g, int weight_kind, double *out);
int oracle_build_rejection(const oracle_graph *g, int weight_kind, double *rej_weight, double *rej_max);

/* Walk W walkers.  Walker i starts at sources[i] (or at sources[i / per_query]
 * when per_query > 0) and has RNG id id_base + i.  paths: W x path_cap,
 * walker-major, padded with -1 (NULL to skip).  lengths: W final length_
 * values (NULL to skip).  counts: visit counts, query-major
 * (query = i / per_query, or 0), NULL to skip.  Returns steps taken in
 * *steps.  threads <= 0 uses all hardware threads.  Returns 0 or a
 * negative error. */
int oracle_walk(const oracle_graph *g, const oracle_walk_desc *d,
                const int32_t *sources, int64_t num_walkers, int64_t per_query,
                int64_t id_base, int32_t *paths, int32_t path_cap,
                int32_t *lengths, int32_t *counts, uint64_t *steps,
                int32_t threads);

/* Same walks through a ring of `ring` interleaved walkers per thread with
 * software prefetch between stages (the step-interleaving scheme of
 * creeper.h:336-541 / uniform_sampling.h:11-45 / alias_sampling.h:69-106).
 * Supports Uniform mode and Static Alias; results equal oracle_walk's. */
int oracle_walk_interleaved(const oracle_graph *g, const oracle_walk_desc *d,
                            const int32_t *sources, int64_t num_walkers, int64_t per_query,
                            int64_t id_base, int32_t *paths, int32_t path_cap,
                            int32_t *lengths, int32_t *counts, uint64_t *steps,
                            int32_t threads, int32_t ring);

/* Algorithmic bytes per step: replays the walks and counts, per move, the
 * distinct 32-byte sectors of each independent random access, the sectors
 * spanned by contiguous row scans, 4 bytes per path write and one 32-byte
 * sector per visit-count update.  Returns total bytes in *bytes. */
/* Accounting of oracle_count_bytes for searches the GPU engine replaces with
 * lookups (bit flags, 0 = the reference's searches): 1 = Node2Vec's
 * neighbour test as one 32-byte hash probe, 2 = MetaPath's label scan as one
 * 32-byte read of label-index offsets. */
void oracle_set_neighbor_accounting(int32_t kind);

int oracle_count_bytes(const oracle_graph *g, const oracle_walk_desc *d,
                       const int32_t *sources, int64_t num_walkers, int64_t per_query,
                       int64_t id_base, int32_t record_paths, int32_t count_visits,
                       uint64_t *bytes, uint64_t *steps, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
