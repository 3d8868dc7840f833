/*
 * trw_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle, never the product).
 *
 * CPU restatement of ThunderRW's sampling path.  Each function names the
 * reference lines it follows (paths relative to the ThunderRW tree).  Built
 * with -ffp-contract=off so every double operation is a single IEEE
 * round-to-nearest operation, as in the reference's x86-64 build.
 */
#include "trw_oracle.h"
#include "philox.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1) { oracle_philox_block(c, k0, k1); }

/* One (walker, step) draw cursor: plays the role of the per-thread sfmt_t of
 * creeper.h:357,449,570, but keyed so every walker's draws are independent of
 * scheduling. */
struct Cursor {
    uint64_t seed, walker;
    uint32_t step, draw = 0, block_base = 0;
    uint32_t cached_block = 0xFFFFFFFFu, buf[4];
    Cursor(uint64_t s, uint64_t w, uint32_t st, uint32_t base = 0)
        : seed(s), walker(w), step(st), block_base(base) {}
    uint32_t u32() {
        uint32_t blk = block_base + (draw >> 2);
        if (blk != cached_block) {
            buf[0] = blk; buf[1] = step; buf[2] = (uint32_t)walker; buf[3] = (uint32_t)(walker >> 32);
            philox(buf, (uint32_t)seed, (uint32_t)(seed >> 32));
            cached_block = blk;
        }
        return buf[draw++ & 3];
    }
};

/* SFMT.h:193-228 */
inline double real1(uint32_t v) { return v * (1.0 / 4294967295.0); }
inline double real2(uint32_t v) { return v * (1.0 / 4294967296.0); }

enum { APP_DEEPWALK = 0, APP_PPR = 1, APP_NODE2VEC = 2, APP_METAPATH = 3, APP_GENERIC = 4 };
enum { MODE_UNIFORM = 0, MODE_STATIC = 1, MODE_DYNAMIC = 2 };
enum { S_UNIFORM = 0, S_ITS = 1, S_ALIAS = 2, S_RS = 3, S_MAXRS = 4 };

constexpr int64_t kMaxTrials = 1 << 20;  /* rejection trials before a walker is stopped */

struct Walker {
    int32_t cur, prev, len;  /* prev = seq_[length_-2] when length_ > 1 */
};

/* Graph::is_neighbor (graph.h:180-199): binary search of the higher-degree
 * endpoint in the lower-degree endpoint's sorted list. */
inline bool is_neighbor(const oracle_graph *g, int32_t u, int32_t v) {
    int64_t du = g->row[u + 1] - g->row[u], dv = g->row[v + 1] - g->row[v];
    if (du < dv) std::swap(u, v);
    const int32_t *nb = g->adj + g->row[v];
    int32_t lo = 0, hi = (int32_t)(g->row[v + 1] - g->row[v]) - 1;
    while (lo <= hi) {
        int32_t mid = lo + ((hi - lo) >> 1);
        if (nb[mid] == u) return true;
        if (nb[mid] > u) hi = mid - 1; else lo = mid + 1;
    }
    return false;
}

struct App {
    int32_t kind, L, S;
    double p_w, q_w, n2v_max, tp;
    const int32_t *schema;
    explicit App(const oracle_walk_desc *d) {
        kind = d->app; L = d->length; S = d->schema_len; schema = d->schema; tp = d->tp;
        /* node2vec.cpp:176-178,227,234: p_ = 1/p, q_ = 1/q, max_ = max(1, q_, p_) */
        p_w = d->p != 0.0 ? 1.0 / d->p : 0.0;
        q_w = d->q != 0.0 ? 1.0 / d->q : 0.0;
        n2v_max = std::max(1.0, std::max(q_w, p_w));
    }
    /* weight hooks: deepwalk.cpp:19-21, ppr.cpp:95-97, node2vec.cpp:182-196,
     * metapath.cpp:22-30, genericwalk.cpp:122-124 */
    double weight(const oracle_graph *g, const Walker &w, int32_t nbr, int64_t eid) const {
        switch (kind) {
        case APP_DEEPWALK: case APP_GENERIC: return g->weight[eid];
        case APP_PPR: return 1.0;
        case APP_NODE2VEC:
            if (w.len == 1) return n2v_max;
            if (nbr == w.prev) return p_w;
            if (is_neighbor(g, w.prev, nbr)) return 1.0;
            return q_w;
        case APP_METAPATH:
            return g->label[eid] != schema[(w.len - 1) % S] ? 0.0 : 1.0;
        }
        return 0.0;
    }
    /* max_weight hooks: deepwalk.cpp:27-29 (5.0), ppr.cpp:103-105 (1.0),
     * node2vec.cpp:202-204 (max_), metapath.cpp:36-38 (1.0), genericwalk.cpp:130-132 (5.0) */
    double max_weight() const {
        switch (kind) {
        case APP_DEEPWALK: case APP_GENERIC: return 5.0;
        case APP_NODE2VEC: return n2v_max;
        default: return 1.0;
        }
    }
    /* update hooks: length_ == l_ (deepwalk.cpp:23-25 and the others), or
     * real1 <= tp for PPR (ppr.cpp:99-101). */
    bool update(uint64_t seed, uint64_t wid, const Walker &w) const {
        if (kind == APP_PPR) {
            Cursor c(seed, wid, (uint32_t)w.len, ORACLE_TERM_BLOCK);
            return real1(c.u32()) <= tp;
        }
        return w.len == L;
    }
};

/* alias_initialization (alias_sampling.h:12-54; same loop as
 * alias_preprocess.cpp:30-73): FIFO small/large queues. */
bool alias_init(double *src, const int32_t *nbrs, oracle_alias_slot *table, int32_t length,
                std::vector<int32_t> &small, std::vector<int32_t> &large) {
    double sum = 0.0;
    for (int32_t j = 0; j < length; ++j) sum += src[j];  /* std::accumulate, left fold */
    double avg = sum / length;
    if (avg == 0.0) return false;
    small.clear(); large.clear();
    for (int32_t j = 0; j < length; ++j) {
        src[j] /= avg;
        if (src[j] < 1) small.push_back(j); else large.push_back(j);
    }
    size_t sh = 0, lh = 0;  /* queue heads; pushes go to the back */
    int32_t index = 0;
    while (sh < small.size() && lh < large.size()) {
        int32_t s = small[sh], l = large[lh];
        table[index++] = {src[s], nbrs[s], nbrs[l]};
        ++sh;
        src[l] = src[l] + src[s] - 1;
        if (src[l] < 1) { ++lh; small.push_back(l); }
    }
    while (sh < small.size()) { int32_t s = small[sh++]; table[index++] = {1.0, nbrs[s], nbrs[s]}; }
    while (lh < large.size()) { int32_t l = large[lh++]; table[index++] = {1.0, nbrs[l], nbrs[l]}; }
    return true;
}

/* Utility::upper_bound_branchless (utility.h:18-27) */
inline int32_t upper_bound_bl(const double *src, int32_t n, double target) {
    const double *base = src;
    while (n > 1) {
        int32_t half = n >> 1;
        base = (base[half] <= target) ? &base[half] : base;
        n -= half;
    }
    return (int32_t)((*base <= target) + (base - src));
}

inline double static_weight(const oracle_graph *g, int weight_kind, int64_t eid) {
    return weight_kind == 0 ? g->weight[eid] : 1.0;
}

struct Scratch {
    std::vector<double> w;
    std::vector<oracle_alias_slot> table;
    std::vector<int32_t> small, large;
};

/* How oracle_count_bytes charges the searches the GPU engine replaces with
 * lookups (bit flags; 0 = the reference's methods): 1 = Node2Vec's neighbour
 * test as one 32-byte probe of a hash set of the edges instead of the binary
 * search (graph.h:180-199); 2 = MetaPath's dynamic ITS from a label index:
 * one 32-byte read of the wanted label's two CSR positions per step instead of
 * the row pair and the label row scan. */
static std::atomic<int> g_neighbor_accounting{0};

extern "C" void oracle_set_neighbor_accounting(int32_t kind) { g_neighbor_accounting.store(kind); }

/* Sector accounting for oracle_count_bytes. */
struct ByteCounter {
    uint64_t bytes = 0;
    std::vector<uint64_t> seen;
    void begin() { seen.clear(); }
    void touch(const void *p) {
        uint64_t s = (uint64_t)(uintptr_t)p >> 5;
        for (uint64_t x : seen) if (x == s) return;
        seen.push_back(s);
        bytes += 32;
    }
    void span(const void *p, size_t nbytes) {
        if (!nbytes) return;
        uint64_t a = (uint64_t)(uintptr_t)p >> 5, b = ((uint64_t)(uintptr_t)p + nbytes - 1) >> 5;
        bytes += (b - a + 1) * 32;
    }
};

/* One walker from admission to completion: the admission of creeper.h:322-331,
 * then repeated gather (creeper.h:179-296 for the dynamic samplers), move
 * (the *_move functions) and update (creeper.h:299-319). */
template <bool kCount>
void walk_one(const oracle_graph *g, const oracle_walk_desc *d, const App &app, uint64_t wid,
              int32_t source, int32_t *path, int32_t path_cap, int32_t *len_out, int32_t *counts,
              uint64_t &steps, Scratch &sc, ByteCounter *bc) {
    Walker w{source, -1, 1};
    if (path && path_cap > 0) path[0] = source;
    const int mode = d->mode, sampler = d->sampler;
    for (;;) {
        const int32_t cur = w.cur;
        const int64_t off = g->row[cur];
        const int32_t deg = (int32_t)(g->row[cur + 1] - off);
        if (kCount) {
            bc->begin();
            if (app.kind == APP_METAPATH && mode == MODE_DYNAMIC && sampler == S_ITS &&
                (g_neighbor_accounting.load(std::memory_order_relaxed) & 2))
                bc->bytes += 32;  /* a label index's two CSR positions of the wanted label, no row pair */
            else
                bc->touch(g->row + cur);
        }
        if (deg == 0) break;  /* a sink: the reference divides by zero here */
        Cursor c(d->seed, wid, (uint32_t)w.len);
        int32_t nxt = -1;
        bool stop = false;
        if (mode == MODE_UNIFORM) {
            /* uniform_move (uniform_sampling.h:47-63) */
            int64_t pos = off + (c.u32() % (uint32_t)deg);
            nxt = g->adj[pos];
            if (kCount) bc->touch(g->adj + pos);
        } else if (mode == MODE_STATIC && sampler == S_ALIAS) {
            /* static_alias_move (alias_sampling.h:147-172) */
            uint32_t p0 = c.u32() % (uint32_t)deg;
            double r1 = real2(c.u32());
            const oracle_alias_slot &s = g->alias[off + p0];
            nxt = r1 <= s.prob ? s.first : s.second;
            if (kCount) bc->touch(&s);
        } else if (mode == MODE_STATIC && sampler == S_ITS) {
            /* static_its_move (inverse_transformation_sampling.h:259-286) */
            const double *wb = g->prefix + off;
            double maxw = wb[deg - 1];
            if (kCount) bc->touch(wb + deg - 1);
            if (maxw == 0.0) { stop = true; }
            else {
                double target = real2(c.u32()) * maxw;
                int32_t sel = upper_bound_bl(wb, deg, target);
                if (kCount) {
                    const double *base = wb; int32_t n = deg;
                    while (n > 1) { int32_t h = n >> 1; bc->touch(base + h); base = (base[h] <= target) ? &base[h] : base; n -= h; }
                    bc->touch(base);
                    bc->touch(g->adj + off + sel);
                }
                nxt = g->adj[off + sel];
            }
        } else if (mode == MODE_STATIC && sampler == S_RS) {
            /* static_rs_move (rejection_sampling.h:334-366) */
            const double *ew = g->rej_weight + off;
            double maxw = g->rej_max[cur];
            if (kCount) bc->touch(g->rej_max + cur);
            uint32_t p0; double r; int64_t t = 0;
            do {
                p0 = c.u32() % (uint32_t)deg;
                r = real2(c.u32()) * maxw;
                if (kCount) bc->touch(ew + p0);
            } while (r > ew[p0] && ++t < kMaxTrials);
            if (t >= kMaxTrials) stop = true;
            else { nxt = g->adj[off + p0]; if (kCount) bc->touch(g->adj + off + p0); }
        } else if (mode == MODE_DYNAMIC && sampler == S_MAXRS) {
            /* creeper.h:648-653 then dynamic_max_weight_rs_move
             * (rejection_sampling.h:368-402) */
            double maxw = app.max_weight();
            uint32_t p0; double r, sel; int64_t t = 0;
            do {
                p0 = c.u32() % (uint32_t)deg;
                int32_t nb = g->adj[off + p0];
                sel = app.weight(g, w, nb, off + p0);
                r = real2(c.u32()) * maxw;
                if (kCount) {
                    bc->touch(g->adj + off + p0);
                    if (app.kind == APP_NODE2VEC && w.len != 1 && nb != w.prev &&
                        (g_neighbor_accounting.load(std::memory_order_relaxed) & 1)) {
                        bc->bytes += 32;  /* one probe of a hash set of the edges */
                    } else if (app.kind == APP_NODE2VEC && w.len != 1 && nb != w.prev) {
                        int32_t u = w.prev, v = nb;
                        bc->touch(g->row + u); bc->touch(g->row + v);
                        int64_t du = g->row[u + 1] - g->row[u], dv = g->row[v + 1] - g->row[v];
                        if (du < dv) std::swap(u, v);
                        const int32_t *list = g->adj + g->row[v];
                        int32_t lo = 0, hi = (int32_t)(g->row[v + 1] - g->row[v]) - 1;
                        while (lo <= hi) {
                            int32_t mid = lo + ((hi - lo) >> 1);
                            bc->touch(list + mid);
                            if (list[mid] == u) break;
                            if (list[mid] > u) hi = mid - 1; else lo = mid + 1;
                        }
                    } else if (app.kind == APP_DEEPWALK || app.kind == APP_GENERIC) {
                        bc->touch(g->weight + off + p0);
                    } else if (app.kind == APP_METAPATH) {
                        bc->touch(g->label + off + p0);
                    }
                }
            } while (r > sel && ++t < kMaxTrials);
            if (t >= kMaxTrials) stop = true;
            else nxt = g->adj[off + p0];
        } else if (mode == MODE_DYNAMIC) {
            /* dynamic_gather (creeper.h:179-296): weights of the whole row via the
             * app hook, then the sampler's per-walker structure. */
            if ((int32_t)sc.w.size() < deg) { sc.w.resize(deg); sc.table.resize(deg); }
            double *wt = sc.w.data();
            for (int32_t i = 0; i < deg; ++i) wt[i] = app.weight(g, w, g->adj[off + i], off + i);
            if (kCount) {
                if (app.kind == APP_METAPATH && sampler == S_ITS &&
                    (g_neighbor_accounting.load(std::memory_order_relaxed) & 2)) {
                    /* charged at the step's start */
                } else if (app.kind == APP_METAPATH) bc->span(g->label + off, (size_t)deg * 4);
                else if (app.kind == APP_DEEPWALK || app.kind == APP_GENERIC) bc->span(g->weight + off, (size_t)deg * 8);
                else if (app.kind == APP_NODE2VEC) bc->span(g->adj + off, (size_t)deg * 4);
            }
            if (sampler == S_ITS) {
                /* creeper.h:261-272, then dynamic_its_move
                 * (inverse_transformation_sampling.h:288-313) */
                for (int32_t x = 1; x < deg; ++x) wt[x] += wt[x - 1];
                if (wt[deg - 1] == 0.0) { stop = true; }
                else {
                    double target = real2(c.u32()) * wt[deg - 1];
                    int32_t sel = upper_bound_bl(wt, deg, target);
                    nxt = g->adj[off + sel];
                    if (kCount) bc->touch(g->adj + off + sel);
                }
            } else if (sampler == S_ALIAS) {
                /* creeper.h:274-282, then dynamic_alias_move (alias_sampling.h:174-199) */
                if (!alias_init(wt, g->adj + off, sc.table.data(), deg, sc.small, sc.large)) {
                    stop = true;
                } else {
                    if (kCount) bc->span(g->adj + off, (size_t)deg * 4);
                    uint32_t p0 = c.u32() % (uint32_t)deg;
                    double r1 = real2(c.u32());
                    const oracle_alias_slot &s = sc.table[p0];
                    nxt = r1 <= s.prob ? s.first : s.second;
                }
            } else if (sampler == S_RS) {
                /* creeper.h:283-293, then dynamic_rs_move (rejection_sampling.h:404-436) */
                double maxw = *std::max_element(wt, wt + deg);
                if (maxw == 0.0) { stop = true; }
                else {
                    uint32_t p0; double r; int64_t t = 0;
                    do {
                        p0 = c.u32() % (uint32_t)deg;
                        r = real2(c.u32()) * maxw;
                    } while (r > wt[p0] && ++t < kMaxTrials);
                    if (t >= kMaxTrials) stop = true;
                    else { nxt = g->adj[off + p0]; if (kCount) bc->touch(g->adj + off + p0); }
                }
            } else {
                stop = true;
            }
        } else {
            stop = true;
        }
        if (stop) break;
        /* the move's bookkeeping (e.g. alias_sampling.h:316-321) */
        w.prev = cur;
        w.cur = nxt;
        if (path && w.len < path_cap) { path[w.len] = nxt; if (kCount) bc->bytes += 4; }
        w.len += 1;
        /* update (creeper.h:299-319) */
        steps += 1;
        if (counts) { __atomic_fetch_add(counts + nxt, 1, __ATOMIC_RELAXED); if (kCount) bc->bytes += 32; }
        if (app.update(d->seed, wid, w)) break;
    }
    if (path) for (int32_t k = w.len; k < path_cap; ++k) path[k] = -1;
    if (len_out) *len_out = w.len;
}

int validate(const oracle_graph *g, const oracle_walk_desc *d) {
    if (!g || !d || !g->row || !g->adj) return -1;
    if (d->mode < 0 || d->mode > 2 || d->sampler < 0 || d->sampler > 4 || d->app < 0 || d->app > 4) return -2;
    /* the walks that would never end in the reference: l_ < 2, tp <= 0 */
    if (d->app != APP_PPR && d->length < 2) return -1;
    if (d->app == APP_PPR && !(d->tp >= 1e-6 && d->tp <= 1.0)) return -1;
    if (d->app == APP_NODE2VEC && !(d->p > 0.0 && d->q > 0.0)) return -1;
    if (d->app == APP_METAPATH && d->mode == MODE_DYNAMIC && d->sampler == S_MAXRS) return -3;
    if (d->mode == MODE_STATIC) {
        if (d->app == APP_NODE2VEC || d->app == APP_METAPATH) return -3;
        if (d->sampler == S_ALIAS && !g->alias) return -4;
        if (d->sampler == S_ITS && !g->prefix) return -4;
        if (d->sampler == S_RS && (!g->rej_weight || !g->rej_max)) return -4;
        if (d->sampler == S_UNIFORM || d->sampler == S_MAXRS) return -2;
    }
    if (d->mode == MODE_DYNAMIC && d->sampler == S_UNIFORM) return -2;
    if ((d->app == APP_DEEPWALK || d->app == APP_GENERIC) && d->mode != MODE_UNIFORM && d->mode != MODE_STATIC && !g->weight) return -4;
    if (d->app == APP_METAPATH && (!g->label || !d->schema || d->schema_len <= 0)) return -4;
    return 0;
}

template <class Fn>
void parallel_for(int64_t n, int32_t threads, Fn fn) {
    int32_t t = threads > 0 ? threads : (int32_t)std::max(1u, std::thread::hardware_concurrency());
    if (n < 4096) t = 1;
    std::atomic<int64_t> next(0);
    const int64_t chunk = 1024;
    auto body = [&](int tid) {
        for (;;) {
            int64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            fn(tid, b, std::min(n, b + chunk));
        }
    };
    if (t == 1) { body(0); return; }
    std::vector<std::thread> pool;
    for (int i = 0; i < t; ++i) pool.emplace_back(body, i);
    for (auto &th : pool) th.join();
}

inline int32_t nthreads(int32_t threads) {
    return threads > 0 ? threads : (int32_t)std::max(1u, std::thread::hardware_concurrency());
}

}  // namespace

extern "C" {

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox(c, key[0], key[1]);
    std::memcpy(out, c, sizeof(c));
}

uint32_t oracle_draw_u32(uint64_t seed, uint64_t walker, uint32_t step, uint32_t d) {
    Cursor c(seed, walker, step);
    uint32_t v = 0;
    for (uint32_t i = 0; i <= d; ++i) v = c.u32();
    return v;
}

/* static_initialization, alias branch (creeper.h:107-130). */
int oracle_build_alias(const oracle_graph *g, int weight_kind, oracle_alias_slot *out) {
    if (!g || !out || (weight_kind == 0 && !g->weight)) return -1;
    std::vector<double> w;
    std::vector<int32_t> small, large;
    for (int32_t v = 0; v < g->n; ++v) {
        int64_t off = g->row[v];
        int32_t deg = (int32_t)(g->row[v + 1] - off);
        if (deg == 0) continue;
        w.resize(deg);
        for (int32_t i = 0; i < deg; ++i) w[i] = static_weight(g, weight_kind, off + i);
        if (!alias_init(w.data(), g->adj + off, out + off, deg, small, large)) {
            /* All-zero rows: the reference leaves the slots uninitialised; here
             * they select each neighbour with equal probability. */
            for (int32_t i = 0; i < deg; ++i) out[off + i] = {1.0, g->adj[off + i], g->adj[off + i]};
        }
    }
    return 0;
}

/* static_initialization, ITS branch (creeper.h:131-151) with its_initialization
 * (inverse_transformation_sampling.h:19-24) = its_preprocess.cpp:21-34. */
int oracle_build_prefix(const oracle_graph *g, int weight_kind, double *out) {
    if (!g || !out || (weight_kind == 0 && !g->weight)) return -1;
    for (int32_t v = 0; v < g->n; ++v) {
        int64_t off = g->row[v];
        int32_t deg = (int32_t)(g->row[v + 1] - off);
        if (deg == 0) continue;
        out[off] = static_weight(g, weight_kind, off);
        for (int32_t i = 1; i < deg; ++i) out[off + i] = out[off + i - 1] + static_weight(g, weight_kind, off + i);
    }
    return 0;
}

/* static_initialization, rejection branch (creeper.h:152-170) with
 * rs_initialization (rejection_sampling.h:12-14) = rejection_preprocess.cpp:24-27. */
int oracle_build_rejection(const oracle_graph *g, int weight_kind, double *rej_weight, double *rej_max) {
    if (!g || !rej_weight || !rej_max || (weight_kind == 0 && !g->weight)) return -1;
    for (int32_t v = 0; v < g->n; ++v) {
        int64_t off = g->row[v];
        int32_t deg = (int32_t)(g->row[v + 1] - off);
        for (int32_t i = 0; i < deg; ++i) rej_weight[off + i] = static_weight(g, weight_kind, off + i);
        rej_max[v] = deg ? *std::max_element(rej_weight + off, rej_weight + off + deg) : 0.0;
    }
    return 0;
}

int oracle_walk(const oracle_graph *g, const oracle_walk_desc *d, const int32_t *sources,
                int64_t num_walkers, int64_t per_query, int64_t id_base, int32_t *paths,
                int32_t path_cap, int32_t *lengths, int32_t *counts, uint64_t *steps,
                int32_t threads) {
    int rc = validate(g, d);
    if (rc) return rc;
    if (num_walkers < 0 || (paths && path_cap <= 0)) return -1;
    const App app(d);
    int32_t nt = nthreads(threads);
    std::vector<uint64_t> tsteps(nt, 0);
    /* visit counts are added with relaxed atomics straight into `counts` */
    parallel_for(num_walkers, nt, [&](int tid, int64_t b, int64_t e) {
        Scratch sc;
        for (int64_t i = b; i < e; ++i) {
            int64_t qi = per_query > 0 ? i / per_query : 0;
            int32_t src = per_query > 0 ? sources[qi] : sources[i];
            int32_t *crow = counts ? counts + (size_t)qi * g->n : nullptr;
            walk_one<false>(g, d, app, (uint64_t)(id_base + i), src,
                            paths ? paths + (size_t)i * path_cap : nullptr, path_cap,
                            lengths ? lengths + i : nullptr, crow, tsteps[tid], sc, nullptr);
        }
    });
    uint64_t total = 0;
    for (uint64_t s : tsteps) total += s;
    if (steps) *steps = total;
    return 0;
}

int oracle_count_bytes(const oracle_graph *g, const oracle_walk_desc *d, const int32_t *sources,
                       int64_t num_walkers, int64_t per_query, int64_t id_base,
                       int32_t record_paths, int32_t count_visits, uint64_t *bytes,
                       uint64_t *steps, int32_t threads) {
    int rc = validate(g, d);
    if (rc) return rc;
    const App app(d);
    int32_t nt = nthreads(threads);
    std::vector<uint64_t> tsteps(nt, 0), tbytes(nt, 0);
    int32_t cap = record_paths ? std::max(1, d->app == APP_PPR ? 1 : d->length) : 0;
    parallel_for(num_walkers, nt, [&](int tid, int64_t b, int64_t e) {
        Scratch sc;
        ByteCounter bc;
        std::vector<int32_t> path(cap > 0 ? cap : 1);
        std::vector<int32_t> dummy(count_visits ? g->n : 1, 0);
        for (int64_t i = b; i < e; ++i) {
            int64_t qi = per_query > 0 ? i / per_query : 0;
            int32_t src = per_query > 0 ? sources[qi] : sources[i];
            walk_one<true>(g, d, app, (uint64_t)(id_base + i), src, cap > 0 ? path.data() : nullptr,
                           cap, nullptr, count_visits ? dummy.data() : nullptr, tsteps[tid], sc, &bc);
        }
        tbytes[tid] += bc.bytes;
    });
    uint64_t ts = 0, tb = 0;
    for (int i = 0; i < nt; ++i) { ts += tsteps[i]; tb += tbytes[i]; }
    if (steps) *steps = ts;
    if (bytes) *bytes = tb;
    return 0;
}

/* Step interleaving: a ring of `ring` walkers per thread; each round runs the
 * stages of every occupied slot before the next stage, issuing prefetches for
 * the next stage's random access (creeper.h:387-399 with
 * uniform_interleaving_move uniform_sampling.h:11-45 and
 * static_alias_interleaving_move alias_sampling.h:221-258; for dynamic mode
 * the ring of creeper.h:543-687: max-weight rejection's first trial
 * position drawn and its neighbour prefetched a stage ahead, as MaxRSFrame
 * does, rs_frame.h:47-83, later trials in place; dynamic ITS with the row
 * pair prefetched and the gather, prefix and search of
 * dynamic_its_interleaving_move in place).  Admission and update follow
 * creeper.h:299-334.  Draws are consumed in the order of walk_one, so the
 * walks are the same. */
int oracle_walk_interleaved(const oracle_graph *g, const oracle_walk_desc *d,
                            const int32_t *sources, int64_t num_walkers, int64_t per_query,
                            int64_t id_base, int32_t *paths, int32_t path_cap,
                            int32_t *lengths, int32_t *counts, uint64_t *steps,
                            int32_t threads, int32_t ring) {
    int rc = validate(g, d);
    if (rc) return rc;
    const bool uniform = d->mode == MODE_UNIFORM;
    const bool alias = d->mode == MODE_STATIC && d->sampler == S_ALIAS;
    const bool maxrs = d->mode == MODE_DYNAMIC && d->sampler == S_MAXRS;
    const bool dits = d->mode == MODE_DYNAMIC && d->sampler == S_ITS;
    if (!uniform && !alias && !maxrs && !dits) return -2;
    if (ring <= 0) ring = 64;
    const App app(d);
    const double maxw = app.max_weight();
    const int32_t nt = nthreads(threads);
    std::vector<uint64_t> tsteps(nt, 0);
    /* static walker chunks per thread, as creeper.h:729-734 */
    auto body = [&](int tid) {
        int64_t chunk = num_walkers / nt;
        int64_t b = tid * chunk, e = tid == nt - 1 ? num_walkers : b + chunk;
        struct Slot {
            bool empty; int64_t idx; Walker w; int64_t pos; int64_t off; int32_t deg; uint32_t u0, u1;
            Cursor c{0, 0, 0};  /* the move's draws (dynamic mode) */
        };
        std::vector<Slot> r(ring);
        std::vector<double> wt;  /* dynamic ITS: the gathered row */
        int64_t next = b;
        uint64_t st = 0;
        auto admit = [&](Slot &s) {
            if (next < e) {
                int64_t i = next++;
                int32_t src = per_query > 0 ? sources[i / per_query] : sources[i];
                s.empty = false; s.idx = i; s.w = Walker{src, -1, 1};
                if (paths) paths[(size_t)i * path_cap] = src;
            } else {
                s.empty = true;
            }
        };
        auto finish = [&](Slot &s) {
            if (paths) for (int32_t k = s.w.len; k < path_cap; ++k) paths[(size_t)s.idx * path_cap + k] = -1;
            if (lengths) lengths[s.idx] = s.w.len;
        };
        for (auto &s : r) admit(s);
        int64_t active = 0;
        for (auto &s : r) active += !s.empty;
        while (active > 0) {
            /* stage 1: draw and prefetch the row pair */
            for (auto &s : r) if (!s.empty) {
                s.c = Cursor(d->seed, (uint64_t)(id_base + s.idx), (uint32_t)s.w.len);
                if (uniform || alias) { s.u0 = s.c.u32(); s.u1 = s.c.u32(); }
                __builtin_prefetch(g->row + s.w.cur);
            }
            /* stage 2: position and prefetch of the adjacency entry / alias slot */
            for (auto &s : r) if (!s.empty) {
                s.off = g->row[s.w.cur];
                s.deg = (int32_t)(g->row[s.w.cur + 1] - s.off);
                if (s.deg == 0) continue;
                if (maxrs) {  /* the first trial's position */
                    s.pos = s.off + (s.c.u32() % (uint32_t)s.deg);
                    __builtin_prefetch(g->adj + s.pos);
                } else if (dits) {
                    __builtin_prefetch(d->app == APP_METAPATH ? (const void *)(g->label + s.off)
                                                              : (const void *)(g->weight + s.off));
                } else {
                    s.pos = s.off + (s.u0 % (uint32_t)s.deg);
                    if (uniform) __builtin_prefetch(g->adj + s.pos); else __builtin_prefetch(g->alias + s.pos);
                }
            }
            /* stage 3: move, then update and refill */
            for (auto &s : r) if (!s.empty) {
                bool done;
                if (s.deg == 0) {
                    done = true;
                } else {
                    int32_t nxt = -1;
                    bool stop = false;
                    if (uniform) nxt = g->adj[s.pos];
                    else if (alias) { const oracle_alias_slot &a = g->alias[s.pos]; nxt = real2(s.u1) <= a.prob ? a.first : a.second; }
                    else if (maxrs) {  /* dynamic_max_weight_rs_move's trials (rejection_sampling.h:368-402) */
                        int64_t t = 0;
                        int64_t pos = s.pos;
                        double sel = app.weight(g, s.w, g->adj[pos], pos);
                        double rr = real2(s.c.u32()) * maxw;
                        while (rr > sel && ++t < kMaxTrials) {
                            pos = s.off + (s.c.u32() % (uint32_t)s.deg);
                            sel = app.weight(g, s.w, g->adj[pos], pos);
                            rr = real2(s.c.u32()) * maxw;
                        }
                        if (t >= kMaxTrials) stop = true;
                        else nxt = g->adj[pos];
                    } else {  /* dynamic ITS: gather, prefix, search (inverse_transformation_sampling.h:288-313) */
                        if ((int32_t)wt.size() < s.deg) wt.resize(s.deg);
                        for (int32_t i = 0; i < s.deg; ++i) wt[i] = app.weight(g, s.w, g->adj[s.off + i], s.off + i);
                        for (int32_t x = 1; x < s.deg; ++x) wt[x] += wt[x - 1];
                        if (wt[s.deg - 1] == 0.0) stop = true;
                        else {
                            const double target = real2(s.c.u32()) * wt[s.deg - 1];
                            nxt = g->adj[s.off + upper_bound_bl(wt.data(), s.deg, target)];
                        }
                    }
                    if (stop) { finish(s); active -= 1; admit(s); active += !s.empty; continue; }
                    s.w.prev = s.w.cur; s.w.cur = nxt;
                    if (paths && s.w.len < path_cap) paths[(size_t)s.idx * path_cap + s.w.len] = nxt;
                    s.w.len += 1;
                    st += 1;
                    if (counts) {
                        int64_t qi = per_query > 0 ? s.idx / per_query : 0;
                        __atomic_fetch_add(counts + (size_t)qi * g->n + nxt, 1, __ATOMIC_RELAXED);
                    }
                    done = app.update(d->seed, (uint64_t)(id_base + s.idx), s.w);
                }
                if (done) { finish(s); active -= 1; admit(s); active += !s.empty; }
            }
        }
        tsteps[tid] = st;
    };
    if (nt == 1) body(0);
    else {
        std::vector<std::thread> pool;
        for (int i = 0; i < nt; ++i) pool.emplace_back(body, i);
        for (auto &th : pool) th.join();
    }
    uint64_t total = 0;
    for (uint64_t s : tsteps) total += s;
    if (steps) *steps = total;
    return 0;
}

}  // extern "C"
