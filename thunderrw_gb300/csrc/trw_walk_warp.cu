// trw_walk_warp.cu -- dynamic-mode walk kernels that gather the whole
// neighbour row every step: dynamic_gather (creeper.h:179-296) followed by
// dynamic ITS (inverse_transformation_sampling.h:147-257,288-313), dynamic
// alias (alias_sampling.h:56-67,108-145,174-199) or dynamic rejection
// (rejection_sampling.h:232-332,404-436).
//
// Each lane owns one walker; the warp walks the row of every active walker in
// turn with coalesced 32-wide loads:
//  * 0/1 weights (MetaPath's label filter, metapath.cpp:22-30): one
//    ballot/popc pass counts the matches, the draw picks rank
//    floor(real2 * count), a second pass finds that match with __fns.  This is
//    exactly the reference's upper bound over the 0/1 prefix sums, whose
//    values are small integers and so exact in any order.
//  * double weights: the prefix sums are chained left to right through warp
//    shuffles in the reference's order (w[x] += w[x-1], creeper.h:261-265), so
//    the total and every prefix value round identically.
//  * rejection: the row maximum (order-independent, so a warp max is exact);
//    the trials then run per lane in parallel, recomputing the hook weight of
//    each probed edge.
//  * alias: lane 0 builds the per-walker alias table in the warp's scratch
//    rows (same FIFO pairing as alias_initialization, alias_sampling.h:12-54),
//    then draws from it.
#include "trw_device.cuh"
#include "trw_internal.h"

namespace trw {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct WSlot {
    int64_t widx, q;
    int32_t cur, prev, len;
    int2 crow, prow;
};

__device__ __forceinline__ void wfinish(const WalkParams &p, WSlot &s) {
    if (p.lengths) p.lengths[s.widx] = s.len;
    if (p.paths) {
        int32_t *row = p.paths + s.widx * (int64_t)p.path_cap;
        for (int32_t k = s.len; k < p.path_cap; ++k) row[k] = -1;
    }
    s.widx = -1;
}

__device__ __forceinline__ void wadmit(const WalkParams &p, WSlot &s, int64_t idx) {
    int64_t q = 0;
    int32_t src;
    if (p.per_query > 0) { q = idx / p.per_query; src = __ldg(p.sources + q); }
    else src = __ldg(p.sources + idx);
    s.widx = idx;
    s.q = q;
    s.len = 1;
    s.prev = -1;
    s.prow = make_int2(0, 0);
    if (p.paths && p.path_cap > 0) p.paths[idx * (int64_t)p.path_cap] = src;
    if (src < 0 || src >= p.g.n) {
        atomicOr(p.error, kErrVertex);
        s.cur = 0;
        wfinish(p, s);
        return;
    }
    s.cur = src;
}

// Hook weight of row entry i of the broadcast walker.
template <int WK>
__device__ __forceinline__ double row_weight(const WalkParams &p, int32_t len, int32_t prev, int2 prow,
                                             int2 crow, int32_t i) {
    const int64_t eid = crow.x + i;
    const int32_t nb = WK == kNode2Vec ? __ldg(p.g.adj + eid) : 0;
    return app_weight<WK>(p, len, prev, prow, nb, eid);
}

// Sequential ITS selection over double weights.  Returns -1 if the total is 0.
template <int WK>
__device__ int32_t its_select_double(const WalkParams &p, int32_t len, int32_t prev, int2 prow, int2 crow,
                                     uint32_t u0) {
    const int lane = threadIdx.x & 31;
    const int32_t deg = crow.y - crow.x;
    double acc = 0.0;
    bool first = true;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        const double w = i < deg ? row_weight<WK>(p, len, prev, prow, crow, i) : 0.0;
        const int m = min(32, deg - base);
        for (int k = 0; k < m; ++k) {
            const double x = __shfl_sync(kFull, w, k);
            acc = first ? x : acc + x;  // P[0] = w[0]; P[i] = P[i-1] + w[i]
            first = false;
        }
    }
    if (acc == 0.0) return -1;
    const double t = acc * real2(u0);  // weight_[last] * dr_ (inverse_transformation_sampling.h:173)
    acc = 0.0;
    first = true;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        const double w = i < deg ? row_weight<WK>(p, len, prev, prow, crow, i) : 0.0;
        const int m = min(32, deg - base);
        double mine = 0.0;
        for (int k = 0; k < m; ++k) {
            const double x = __shfl_sync(kFull, w, k);
            acc = first ? x : acc + x;
            first = false;
            if (lane == k) mine = acc;
        }
        const unsigned hit = __ballot_sync(kFull, lane < m && mine > t);
        if (hit) return base + __ffs(hit) - 1;
    }
    return deg;  // unreachable for a positive total
}

// Label rows are read as 16-byte words from the aligned element a0 =
// crow.x & ~3 (the label array is padded to a multiple of 4 elements), in
// tiles of 128 elements (one int4 per lane) and kLabelUnroll tiles in flight
// per lane.  Tiles are counted in at most kLabelGroups groups of whole load
// rounds whose match counts stay in shared memory, so the selection pass
// re-reads one group instead of the row.
constexpr int kLabelUnroll = 8;
constexpr int kLabelGroups = 256;

// Matches of the 4 labels in v (elements e..e+3 counted from a0) that lie in
// the row; bit k = element e + k.
__device__ __forceinline__ uint32_t label_bits(int4 v, int32_t e, int32_t lo, int32_t span, int32_t want) {
    uint32_t b = 0;
    b |= (v.x == want && e + 0 >= lo && e + 0 < span) ? 1u : 0u;
    b |= (v.y == want && e + 1 >= lo && e + 1 < span) ? 2u : 0u;
    b |= (v.z == want && e + 2 >= lo && e + 2 < span) ? 4u : 0u;
    b |= (v.w == want && e + 3 >= lo && e + 3 < span) ? 8u : 0u;
    return b;
}

// ITS over 0/1 label weights: the reference's upper bound over the 0/1
// prefix sums picks match number floor(count * real2) in row order.
// gc: this warp's kLabelGroups counters in shared memory.
__device__ int32_t its_select_label(const WalkParams &p, int32_t len, int2 crow, uint32_t u0, uint32_t *gc) {
    const int lane = threadIdx.x & 31;
    const int32_t want = p.schema[(len - 1) % p.schema_len];
    const int32_t a0 = crow.x & ~3;
    const int32_t lo = crow.x - a0;   // first row element, counted from a0
    const int32_t span = crow.y - a0; // one past the last
    const int32_t ntiles = (span + 127) >> 7;
    constexpr int32_t kRound = kLabelUnroll * kLabelGroups;
    const int32_t gs = kLabelUnroll * ((ntiles + kRound - 1) / kRound);  // tiles per group
    const int4 *base = reinterpret_cast<const int4 *>(p.g.label + a0);
    uint32_t total = 0;
    for (int32_t t0 = 0; t0 < ntiles; t0 += kLabelUnroll) {
        int4 v[kLabelUnroll];
#pragma unroll
        for (int u = 0; u < kLabelUnroll; ++u) {
            const int32_t e = ((t0 + u) << 7) + (lane << 2);
            v[u] = e < span ? __ldg(base + ((t0 + u) << 5) + lane) : make_int4(0, 0, 0, 0);
        }
        uint32_t c = 0;
#pragma unroll
        for (int u = 0; u < kLabelUnroll; ++u)
            c += __popc(label_bits(v[u], ((t0 + u) << 7) + (lane << 2), lo, span, want));
        const uint32_t tot = __reduce_add_sync(kFull, c);
        if (lane == 0) {
            const int32_t g = t0 / gs;
            gc[g] = (t0 % gs == 0 ? 0u : gc[g]) + tot;
        }
        total += tot;
    }
    if (total == 0) return -1;
    const uint32_t m = (uint32_t)((double)total * real2(u0));  // floor of P[last] * dr_
    __syncwarp();
    // group holding match m: lane l sums groups 8l .. 8l+7, scan over lanes
    const int32_t ng = (ntiles + gs - 1) / gs;
    uint32_t own[kLabelGroups / 32];
    uint32_t lsum = 0;
#pragma unroll
    for (int k = 0; k < kLabelGroups / 32; ++k) {
        const int32_t g = lane * (kLabelGroups / 32) + k;
        own[k] = g < ng ? gc[g] : 0u;
        lsum += own[k];
    }
    __syncwarp();  // gc is rewritten by the next walker's count pass
    uint32_t incl = lsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    const unsigned hit = __ballot_sync(kFull, incl > m);
    const int src = __ffs(hit) - 1;
    int32_t grp = 0;
    uint32_t before = 0;
    if (lane == src) {
        before = incl - lsum;
        int kk = -1;
#pragma unroll
        for (int k = 0; k < kLabelGroups / 32; ++k) {  // constant indices keep own[] in registers
            if (kk < 0) {
                if (before + own[k] > m) kk = k;
                else before += own[k];
            }
        }
        grp = lane * (kLabelGroups / 32) + kk;
    }
    grp = __shfl_sync(kFull, grp, src);
    before = __shfl_sync(kFull, before, src);
    const int32_t tend = min((grp + 1) * gs, ntiles);
    for (int32_t t = grp * gs; t < tend; ++t) {
        const int32_t e = (t << 7) + (lane << 2);
        const int4 v = e < span ? __ldg(base + (t << 5) + lane) : make_int4(0, 0, 0, 0);
        const uint32_t b = label_bits(v, e, lo, span, want);
        const uint32_t c = __popc(b);
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += y;
        }
        const uint32_t tile = __shfl_sync(kFull, x, 31);
        if (before + tile > m) {
            const uint32_t r = m - before;  // rank inside this tile
            const bool mine = r >= x - c && r < x;
            const unsigned who = __ballot_sync(kFull, mine);
            int32_t sel = 0;
            if (mine) sel = a0 + e + (int32_t)__fns(b, 0, (int)(r - (x - c)) + 1) - crow.x;
            return __shfl_sync(kFull, sel, __ffs(who) - 1);
        }
        before += tile;
    }
    return -1;  // unreachable: group grp holds match m
}

// Row maximum of the hook weights (exact in any order).
template <int WK>
__device__ double row_max(const WalkParams &p, int32_t len, int32_t prev, int2 prow, int2 crow) {
    const int lane = threadIdx.x & 31;
    const int32_t deg = crow.y - crow.x;
    double mx = 0.0;
    bool any = false;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        if (i < deg) {
            const double w = row_weight<WK>(p, len, prev, prow, crow, i);
            mx = any ? fmax(mx, w) : w;
            any = true;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const double other = __shfl_xor_sync(kFull, mx, o);
        const bool oany = __shfl_xor_sync(kFull, any, o);
        if (oany) { mx = any ? fmax(mx, other) : other; any = true; }
    }
    return mx;
}

// Dynamic alias for the broadcast walker: builds the table in `tab` (deg
// slots) from the raw weights staged in `raw` (deg slots), then draws.
// Returns the chosen vertex or -1 when the average weight is 0.
//
// Slot j of the table always belongs to the j-th index of the stable
// small-then-large partition: the small queue of alias_initialization is the
// initial smalls followed by the larges in the order they turn small, and the
// leftovers are written in queue order, so each pop writes slot j = pop
// number j.  tab[j].first holds that index until the slot is final, and a
// large that turns small parks its value in its own (not yet written) slot.
template <int WK>
__device__ int32_t alias_draw(const WalkParams &p, int32_t len, int32_t prev, int2 prow, int2 crow,
                              AliasSlot *raw, AliasSlot *tab, uint32_t u0, uint32_t u1) {
    const int lane = threadIdx.x & 31;
    const int32_t deg = crow.y - crow.x;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        if (i < deg) raw[i].prob = row_weight<WK>(p, len, prev, prow, crow, i);
    }
    __syncwarp();
    double avg = 0.0;
    if (lane == 0) {
        double sum = 0.0;
        for (int32_t j = 0; j < deg; ++j) sum += raw[j].prob;  // std::accumulate
        avg = sum / deg;
    }
    avg = __shfl_sync(kFull, avg, 0);
    if (avg == 0.0) return -1;
    // stable partition by (w/avg < 1): smalls first
    uint32_t ns = 0;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        ns += __popc(__ballot_sync(kFull, i < deg && raw[i].prob / avg < 1));
    }
    uint32_t sb = 0, lb = ns;
    for (int32_t base = 0; base < deg; base += 32) {
        const int32_t i = base + lane;
        const bool valid = i < deg;
        const double sc = valid ? raw[i].prob / avg : 0.0;
        const bool small = valid && sc < 1;
        const unsigned bs = __ballot_sync(kFull, small), bl = __ballot_sync(kFull, valid && !small);
        if (valid) {
            const uint32_t pos = small ? sb + __popc(bs & lanemask_lt()) : lb + __popc(bl & lanemask_lt());
            tab[pos].prob = sc;
            tab[pos].first = i;
        }
        sb += __popc(bs);
        lb += __popc(bl);
    }
    __syncwarp();
    if (lane == 0) {
        const int32_t *nb = p.g.adj + crow.x;
        const uint32_t nl = (uint32_t)deg - ns;
        uint32_t sp = 0, c = 0;
        double vl = nl ? tab[ns].prob : 0.0;
        while (sp < ns + c && c < nl) {
            const double vs = tab[sp].prob;
            const int32_t si = tab[sp].first;
            const int32_t li = tab[ns + c].first;
            tab[sp].prob = vs;
            tab[sp].first = __ldg(nb + si);
            tab[sp].second = __ldg(nb + li);
            ++sp;
            vl = vl + vs - 1;  // src[l] + src[s] - 1 (alias_sampling.h:187)
            if (vl < 1) {
                tab[ns + c].prob = vl;
                ++c;
                if (c < nl) vl = tab[ns + c].prob;
            }
        }
        for (uint32_t j = sp; j < (uint32_t)deg; ++j) {
            const int32_t v = __ldg(nb + tab[j].first);
            tab[j].prob = 1.0;
            tab[j].first = v;
            tab[j].second = v;
        }
    }
    __syncwarp();
    const uint32_t p0 = u0 % (uint32_t)deg;
    const AliasSlot s = tab[p0];
    return real2_le(u1, s.prob) ? s.first : s.second;
}

template <int S, int U, int WK>
__global__ void __launch_bounds__(kThreadBlock) walk_warp(const WalkParams p, int persistent) {
    const int lane = threadIdx.x & 31;
    const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    __shared__ uint32_t label_groups[WK == kLabelSchema ? kThreadBlock / 32 : 1][kLabelGroups];
    uint32_t *gc = label_groups[WK == kLabelSchema ? threadIdx.x >> 5 : 0];
    AliasSlot *raw = nullptr, *tab = nullptr;
    if (S == kAlias) {
        raw = p.alias_scratch + warp_id * p.alias_scratch_stride;
        tab = raw + p.alias_scratch_stride / 2;
    }
    WSlot s;
    s.widx = -1;
    uint64_t steps = 0;
    unsigned long long res_next = 0, res_end = 0;
    bool drained = false;
    if (!persistent) {  // plain form: one fixed group of 32 walkers per warp
        const int64_t idx = warp_id * 32 + lane;
        if (idx < p.num_walkers) wadmit(p, s, idx);
        drained = true;
    }
    for (;;) {
        unsigned need = __ballot_sync(kFull, s.widx < 0);
        while (need && !drained) {
            if (res_next >= res_end) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(p.queue_head, 64ull);
                b = __shfl_sync(kFull, b, 0);
                if (b >= (unsigned long long)p.num_walkers) { drained = true; break; }
                res_next = b;
                res_end = min(b + 64ull, (unsigned long long)p.num_walkers);
            }
            const unsigned avail = (unsigned)min(res_end - res_next, 32ull);
            const unsigned rank = __popc(need & lanemask_lt());
            const bool mine = ((need >> lane) & 1u) && rank < avail;
            if (mine) wadmit(p, s, (int64_t)(res_next + rank));
            res_next += min((unsigned)__popc(need), avail);
            need &= ~__ballot_sync(kFull, mine);
        }
        unsigned act = __ballot_sync(kFull, s.widx >= 0);
        if (!act) break;
        if (s.widx >= 0) s.crow = __ldg(p.g.rows + s.cur);
        int32_t my_nxt = -1;   // chosen vertex, -1 = the walker stops
        double my_max = 0.0;   // rejection: row maximum
        uint4 my_rnd = make_uint4(0, 0, 0, 0);
        if (s.widx >= 0) my_rnd = draw_block(p.seed, (uint64_t)(p.id_base + s.widx), (uint32_t)s.len, 0);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const int2 crow = make_int2(__shfl_sync(kFull, s.crow.x, j), __shfl_sync(kFull, s.crow.y, j));
            const int32_t len = __shfl_sync(kFull, s.len, j);
            const int32_t prev = __shfl_sync(kFull, s.prev, j);
            const int2 prow = make_int2(__shfl_sync(kFull, s.prow.x, j), __shfl_sync(kFull, s.prow.y, j));
            const uint32_t u0 = __shfl_sync(kFull, my_rnd.x, j);
            const uint32_t u1 = __shfl_sync(kFull, my_rnd.y, j);
            const int32_t deg = crow.y - crow.x;
            if (deg <= 0) continue;  // stops (my_nxt stays -1)
            if (S == kITS) {
                const int32_t sel = WK == kLabelSchema ? its_select_label(p, len, crow, u0, gc)
                                                       : its_select_double<WK>(p, len, prev, prow, crow, u0);
                if (lane == j && sel >= 0) my_nxt = __ldg(p.g.adj + crow.x + sel);
            } else if (S == kRejection) {
                const double mx = row_max<WK>(p, len, prev, prow, crow);
                if (lane == j) my_max = mx;
            } else {
                const int32_t v = alias_draw<WK>(p, len, prev, prow, crow, raw, tab, u0, u1);
                if (lane == j) my_nxt = v;
                __syncwarp();
            }
        }
        if (S == kRejection && s.widx >= 0 && my_max != 0.0) {  // a zero row maximum stops the walker (creeper.h:283-293)
            // trials of dynamic_rs_move (rejection_sampling.h:404-436), per lane
            const int32_t deg = s.crow.y - s.crow.x;
            if (deg > 0) {
                DrawCursor c(p.seed, (uint64_t)(p.id_base + s.widx), (uint32_t)s.len, my_rnd);
                uint32_t trials = 0;
                int32_t p0;
                for (;;) {
                    p0 = (int32_t)(c.next() % (uint32_t)deg);
                    const double y = real2(c.next()) * my_max;
                    const double w = row_weight<WK>(p, s.len, s.prev, s.prow, s.crow, p0);
                    if (y <= w) break;
                    if (++trials >= kMaxTrials) break;
                }
                if (trials >= kMaxTrials) atomicOr(p.error, kErrTrials);
                else my_nxt = __ldg(p.g.adj + s.crow.x + p0);
            }
        }
        if (s.widx >= 0) {
            if (my_nxt < 0) {
                wfinish(p, s);  // zero total weight: terminated without a step (creeper.h:267-292)
            } else {
                s.prev = s.cur;
                s.prow = s.crow;
                s.cur = my_nxt;
                if (p.paths && s.len < p.path_cap) p.paths[s.widx * (int64_t)p.path_cap + s.len] = my_nxt;
                s.len += 1;
                steps += 1;
                record_visit(p, s.q, my_nxt);
                if (app_update<U>(p, (uint64_t)(p.id_base + s.widx), s.len)) wfinish(p, s);
            }
        }
    }
    unsigned long long v = steps;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (lane == 0 && v) atomicAdd(p.steps, v);
}

template <class K>
int max_occupancy(K kernel) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kThreadBlock, 0) != cudaSuccess || n <= 0) n = 1;
    return n;
}

template <int S, int U, int WK>
cudaError_t launch_kind(const WalkParams &p, const LaunchShape &shape, cudaStream_t st) {
    // Dynamic alias always runs persistent: its grid is capped by the scratch
    // tables provisioned (one per warp), and the queue covers every walker.
    const bool persistent = shape.engine != kEnginePlain || S == kAlias;
    int64_t grid;
    if (!persistent) {
        grid = (p.num_walkers + kThreadBlock - 1) / kThreadBlock;
    } else {
        static const int max_occ = max_occupancy(walk_warp<S, U, WK>);
        const int per_sm = shape.ctas_per_sm > 0 ? min(shape.ctas_per_sm, max_occ) : max_occ;
        grid = (int64_t)shape.num_sms * per_sm;
        const int64_t useful = (p.num_walkers + kThreadBlock - 1) / kThreadBlock;
        if (useful < grid) grid = useful;
        if (S == kAlias) {
            const int64_t cap = shape.max_warps / (kThreadBlock / 32);
            if (cap < grid) grid = cap;
        }
    }
    if (grid <= 0) return cudaSuccess;
    walk_warp<S, U, WK><<<(unsigned)grid, kThreadBlock, 0, st>>>(p, persistent ? 1 : 0);
    return cudaGetLastError();
}

template <int S>
cudaError_t launch_sampler(const WalkParams &p, int update, int wk, const LaunchShape &shape, cudaStream_t st) {
    if (update == kGeometric) {
        if (wk == kUnitWeight) return launch_kind<S, kGeometric, kUnitWeight>(p, shape, st);
        return cudaErrorInvalidValue;
    }
    switch (wk) {
    case kEdgeWeight: return launch_kind<S, kFixedLength, kEdgeWeight>(p, shape, st);
    case kNode2Vec: return launch_kind<S, kFixedLength, kNode2Vec>(p, shape, st);
    case kLabelSchema: return launch_kind<S, kFixedLength, kLabelSchema>(p, shape, st);
    default: return launch_kind<S, kFixedLength, kUnitWeight>(p, shape, st);
    }
}

}  // namespace

cudaError_t launch_walk_warp(const WalkParams &p, int sampler, int update, int weight_kind,
                             const LaunchShape &shape, cudaStream_t st) {
    switch (sampler) {
    case kITS: return launch_sampler<kITS>(p, update, weight_kind, shape, st);
    case kAlias: return launch_sampler<kAlias>(p, update, weight_kind, shape, st);
    case kRejection: return launch_sampler<kRejection>(p, update, weight_kind, shape, st);
    }
    return cudaErrorInvalidValue;
}

int64_t warp_engine_warps(const WalkParams &p, const LaunchShape &shape) {
    // upper bound on the warps of a dynamic-alias launch (one scratch table each)
    int64_t grid = (int64_t)shape.num_sms * 8;
    const int64_t useful = (p.num_walkers + kThreadBlock - 1) / kThreadBlock;
    if (useful < grid) grid = useful;
    return grid * (kThreadBlock / 32);
}

}  // namespace trw
