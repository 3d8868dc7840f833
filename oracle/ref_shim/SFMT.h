/*
 * SFMT.h shim -- TEST INFRASTRUCTURE ONLY.
 *
 * Placed first on the include path when the reference's own sampler code is
 * compiled into the parity harness (oracle/ref_harness.cpp).  It keeps the
 * SFMT API the reference calls (sfmt_t, sfmt_init_gen_rand,
 * sfmt_genrand_uint32/real1/real2; SFMT.h:125-228 of SFMT 1.5.1) but draws
 * from the counter-based Philox stream keyed by (seed, walker, step, draw#),
 * so every draw of every walker is attributed the same way as in the GPU
 * kernels.  The u32 -> double conversions are SFMT's own
 * (SFMT.h:193-228): v * (1/(2^32-1)) and v * 2^-32.
 */
#ifndef TRW_SFMT_SHIM_H
#define TRW_SFMT_SHIM_H

#include <stdint.h>
#include "../philox.h"

typedef struct {
    uint64_t seed;
    uint64_t walker;
    uint32_t step;
    uint32_t draw;
    uint32_t block_base;
} sfmt_t;

static inline void sfmt_init_gen_rand(sfmt_t *s, uint32_t seed) {
    s->seed = seed; s->walker = 0; s->step = 0; s->draw = 0; s->block_base = 0;
}

static inline uint32_t sfmt_genrand_uint32(sfmt_t *s) {
    uint32_t c[4] = {s->block_base + (s->draw >> 2), s->step, (uint32_t)s->walker,
                     (uint32_t)(s->walker >> 32)};
    oracle_philox_block(c, (uint32_t)s->seed, (uint32_t)(s->seed >> 32));
    return c[s->draw++ & 3];
}

static inline double sfmt_to_real1(uint32_t v) { return v * (1.0 / 4294967295.0); }
static inline double sfmt_to_real2(uint32_t v) { return v * (1.0 / 4294967296.0); }
static inline double sfmt_genrand_real1(sfmt_t *s) { return sfmt_to_real1(sfmt_genrand_uint32(s)); }
static inline double sfmt_genrand_real2(sfmt_t *s) { return sfmt_to_real2(sfmt_genrand_uint32(s)); }

#endif
