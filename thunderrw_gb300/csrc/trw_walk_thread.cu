// trw_walk_thread.cu -- walk kernels where each lane owns its walkers:
// Uniform (uniform_sampling.h), static Alias (alias_sampling.h:69-106,147-172),
// static ITS (inverse_transformation_sampling.h:36-145,259-286), static
// Rejection (rejection_sampling.h:28-137,334-366) and dynamic max-weight
// Rejection (rejection_sampling.h:139-230,368-402 with MaxRSFrame,
// rs_frame.h:47-83), under the Gather-Move-Update loop of creeper.h:336-541.
//
// Persistent engine: a grid of (SM count x CTAs/SM) CTAs; every lane keeps R
// walkers in flight (the GPU analogue of the reference's RING_SIZE ring,
// types.h:21) and runs each step stage for all R walkers before the next
// stage, so a lane has R independent random loads outstanding per stage.  A
// lane whose walker finishes takes the next walker id from its warp's
// reservoir, refilled by one atomicAdd per kChunk walkers on a global queue
// head (the admission of creeper.h:321-332).
//
// Plain engine: one thread per walker, walker = global thread id, no refill.
#include "trw_device.cuh"
#include "trw_internal.h"

namespace trw {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct Slot {
    int64_t widx;   // walker index in the call, -1 = empty
    int32_t q;      // query of the walker (visit counts; the API keeps queries < 2^31)
    int32_t cur, prev, len;
    int2 crow, prow;  // row pairs of cur and prev
};

// Path entries of the CTA's ring slots being gathered into groups of four
// (WalkParams::path_vec): component c of slot r of thread t at
// [(c * R + r) * kThreadBlock + t], so a warp's accesses hit distinct banks.
template <int R>
__device__ __forceinline__ int32_t *path_stage() {
    __shared__ int32_t stage[4 * R * kThreadBlock];
    return stage;
}

// Path entry k of ring slot r's walker.  With p.path_vec the entries of each
// group of four gather in shared memory and leave as one 16-byte store: a
// walker's path row then fills whole sectors instead of 4-byte pieces that
// leave L2 half written (each such sector costs DRAM a read-modify-write).
template <bool kVec, int R>
__device__ __forceinline__ void path_put(const WalkParams &p, const Slot &s, int r, int32_t k, int32_t v) {
    if (!kVec || !p.path_vec) {
        p.paths[s.widx * (int64_t)p.path_cap + k] = v;
        return;
    }
    int32_t *st = path_stage<R>() + r * kThreadBlock + threadIdx.x;
    const int c = k & 3;
    if (c < 3) {
        st[c * R * kThreadBlock] = v;
        return;
    }
    const int4 g = make_int4(st[0], st[R * kThreadBlock], st[2 * R * kThreadBlock], v);
    *reinterpret_cast<int4 *>(p.paths + s.widx * (int64_t)p.path_cap + (k - 3)) = g;
}

// The end of slot r's path: the pending group, then -1 up to path_cap
// (out of line: walks that stop early are rare, and inlined at every finish
// this code costs the step loop registers).
template <bool kVec, int R>
__device__ __noinline__ void finish_path(const WalkParams &p, int64_t widx, int32_t len, int r) {
    int32_t *row = p.paths + widx * (int64_t)p.path_cap;
    int32_t k = len;
    if (!kVec || !p.path_vec) {
        for (; k < p.path_cap; ++k) row[k] = -1;
        return;
    }
    if (k >= p.path_cap) return;
    if (k & 3) {  // the pending group: its gathered entries below k, then -1
        const int c = k & 3;
        const int32_t *st = path_stage<R>() + r * kThreadBlock + threadIdx.x;
        const int4 g = make_int4(st[0], c > 1 ? st[R * kThreadBlock] : -1, c > 2 ? st[2 * R * kThreadBlock] : -1, -1);
        *reinterpret_cast<int4 *>(row + (k & ~3)) = g;
        k = (k + 3) & ~3;
    }
    for (; k < p.path_cap; k += 4) *reinterpret_cast<int4 *>(row + k) = make_int4(-1, -1, -1, -1);
}

// kVec: gather path entries (only the static alias walks: with the graph in
// L2 their DRAM traffic is the paths; DeepWalk on Chung-Lu 2^18 0.270 ->
// 0.245 ms, 26.0 -> 20.7 B/step.  Node2Vec and MetaPath lost 2 % to the
// registers it takes.)
template <int S>
__host__ __device__ constexpr bool path_gather() { return S == kAlias; }

template <bool kVec, int R>
__device__ __forceinline__ void finish(const WalkParams &p, Slot &s, int r) {
    if (p.lengths) p.lengths[s.widx] = s.len;
    if (p.paths) {
        if (kVec) {
            if (s.len < p.path_cap) finish_path<kVec, R>(p, s.widx, s.len, r);
        } else {
            int32_t *row = p.paths + s.widx * (int64_t)p.path_cap;
            for (int32_t k = s.len; k < p.path_cap; ++k) row[k] = -1;
        }
    }
    s.widx = -1;
}

// Sampler S moving through DevGraph::fat or DevGraph::lab_fat when they are
// there: the slot then carries the current vertex's row pair, or for the
// label index its first step's block of positions (read here for the
// source).
template <int S, int R>
__device__ __forceinline__ void admit(const WalkParams &p, Slot &s, int r, int64_t idx) {
    int64_t q = 0;
    int32_t src;
    if (p.per_query > 0) { q = idx / p.per_query; src = __ldg(p.sources + q); }
    else src = __ldg(p.sources + idx);
    s.widx = idx;
    s.q = (int32_t)q;
    s.len = 1;
    s.prev = -1;
    s.prow = make_int2(0, 0);
    if (p.paths && p.path_cap > 0) path_put<path_gather<S>(), R>(p, s, r, 0, src);
    if (src < 0 || src >= p.g.n) {  // rejected here so no kernel reads outside the graph
        atomicOr(p.error, kErrVertex);
        s.cur = 0;
        finish<path_gather<S>(), R>(p, s, r);
        return;
    }
    s.cur = src;
    if ((S == kUniform || S == kMaxRejection) && p.g.fat) s.crow = __ldg(p.g.rows + src);
    if (S == kLabelIndex && p.g.lab_fat) {
        const int32_t want = p.schema[0];
        s.crow = make_int2(0, 0);  // a label no edge has: no match
        if (want >= 0 && want < p.g.lab_k) {
            const int32_t *off = p.g.lab_off + (int64_t)src * (p.g.lab_k + 1) + want;
            s.crow = make_int2(__ldg(off), __ldg(off + 1));
        }
    }
}

__device__ __forceinline__ AliasSlot load_alias(const AliasSlot *a) {
    const int4 v = __ldg(reinterpret_cast<const int4 *>(a));
    AliasSlot s;
    s.prob = __hiloint2double(v.y, v.x);
    s.first = v.z;
    s.second = v.w;
    return s;
}

// A sparse visit-count insert in flight (kSparse kernels), advanced once per
// ring round so that no round trip stalls the warp:
//  * recording a visit (end of round i) issues an L2 load of the key in the
//    vertex's home slot;
//  * at round i+1, right after the row-pair loads are issued, the load result
//    is consumed: our key -> add the count (fire-and-forget); empty -> claim
//    it with a CAS, adding all but one of the visits speculatively (a slot's
//    count holds its visits minus the first, which its claim implies; for a
//    single visit, the common case, the claim is the only atomic); another
//    key -> load the next slot (linear probing, as table_add);
//  * the CAS result is consumed when the slot records its next visit, a whole
//    dependent-load chain later: a race lost to the same vertex adds the one
//    visit the claim would have implied; one lost to another vertex takes the
//    speculative part back and probes on.  (Each query's number of distinct
//    vertices is counted from its table after the walk.)
struct PendingInsert {
    int32_t q;      // query of the table, -1 = nothing pending
    uint32_t h;     // slot being examined
    int32_t key;    // vertex + 1
    int32_t old;    // key found in slot h (by the load or the CAS)
    // bits 0-5: visits merged by the warp (1..32); bit 6: `old` came from a
    // CAS of slot h whose count was already added; bits 7-31: slots probed
    // (a table is at most 80 % full, so probe runs stay far below 2^25; a
    // longer one is reported as a full table)
    uint32_t meta;
};

constexpr uint32_t kIncMask = 0x3Fu;
constexpr uint32_t kCasBit = 0x40u;
constexpr uint32_t kProbeLimit = (1u << 25) - 1u;

// One insert record per ring slot: a record is reused when its slot records
// its next visit, a whole dependent-load chain after its CAS was issued, so
// the CAS result has normally arrived.  (Two records per slot cost seven
// more registers: 5 instead of 6 CTAs/SM and a 4 % slower C2 walk on GB300.)
constexpr int kInsertDepth = 1;

__device__ __forceinline__ int32_t *table_of(const WalkParams &p, int32_t q) {
    return p.table + ((int64_t)q << (p.table_bits + 1));
}

// Advances the insert by one stage; with `blocking` it runs to completion.
__device__ __forceinline__ void resolve(const WalkParams &p, PendingInsert &pi, bool blocking) {
    if (pi.q < 0) return;
    const uint32_t mask = (1u << p.table_bits) - 1u;
    int32_t *t = table_of(p, pi.q);
    const int32_t inc = (int32_t)(pi.meta & kIncMask);
    for (;;) {
        if (pi.meta & kCasBit) {
            if (pi.old == 0) { pi.q = -1; return; }  // claimed: its first visit is implied
            if (pi.old == pi.key) {                  // another warp claimed it for this vertex
                atomicAdd(t + mask + 1 + pi.h, 1);
                pi.q = -1;
                return;
            }
            if (inc > 1) atomicAdd(t + mask + 1 + pi.h, 1 - inc);  // lost it to another vertex
        } else {
            if (pi.old == pi.key) {
                atomicAdd(t + mask + 1 + pi.h, inc);
                pi.q = -1;
                return;
            }
            if (pi.old == 0) {
                pi.old = atomicCAS(t + pi.h, 0, pi.key);
                if (inc > 1) atomicAdd(t + mask + 1 + pi.h, inc - 1);  // speculative
                pi.meta |= kCasBit;
                if (!blocking) return;
                continue;
            }
        }
        const uint32_t probes = pi.meta >> 7;
        if (probes >= kProbeLimit || probes >= mask) {  // every slot holds another vertex
            atomicOr(p.error, kErrCapacity);
            pi.q = -1;
            return;
        }
        pi.meta = (pi.meta & kIncMask) + ((probes + 1) << 7);  // cas bit cleared
        pi.h = (pi.h + 1) & mask;
        pi.old = ldcg_keep(t + pi.h);
        if (!blocking) return;
    }
}

__device__ __forceinline__ void start_insert(const WalkParams &p, PendingInsert &pi, int32_t q, int32_t v, int inc) {
    if (pi.q >= 0) resolve(p, pi, true);  // filled a visit ago: normally already settled
    pi.q = q;
    pi.h = ((uint32_t)v * 0x9E3779B1u) >> (32 - p.table_bits);
    pi.key = v + 1;
    pi.meta = (uint32_t)inc;
    pi.old = ldcg_keep(table_of(p, pi.q) + pi.h);
}

// One step for each of the R slots, stage by stage.  kSparse: visits go to
// the per-query tables through the pipelined inserts in `pend`.
template <int S, int U, int WK, int R, bool kSparse>
__device__ __forceinline__ void step_ring(const WalkParams &p, Slot (&s)[R], uint64_t &steps,
                                          PendingInsert (&pend)[R][kInsertDepth]) {
    const DevGraph &g = p.g;
    // uniform and max-weight rejection moves through the adjacency with row
    // pairs, label-index moves through the index with the next positions: the
    // slot already holds the current row (block), and the entry a move takes
    // brings the next one with its vertex
    const bool fat = ((S == kUniform || S == kMaxRejection) && g.fat != nullptr) ||
                     (S == kLabelIndex && g.lab_fat != nullptr);
    int32_t nxt[R];
    int2 nrow[R];
    bool moved[R];
    uint4 rnd[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        moved[r] = false;
        nxt[r] = 0;
        // the label index holds CSR positions itself: no row pair to read
        if (S != kLabelIndex && !fat && s[r].widx >= 0) s[r].crow = __ldg(g.rows + s[r].cur);
    }
    if (kSparse) {  // while the row pairs are in flight
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < kInsertDepth; ++k)
                if (pend[r][k].q >= 0 && !(pend[r][k].meta & kCasBit)) resolve(p, pend[r][k], false);
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (s[r].widx >= 0) rnd[r] = draw_block(p.seed, (uint64_t)(p.id_base + s[r].widx), (uint32_t)s[r].len, 0);

    if (S == kUniform) {
        // uniform_interleaving_move (uniform_sampling.h:11-45)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (s[r].widx < 0) continue;
            const int32_t deg = s[r].crow.y - s[r].crow.x;
            if (deg <= 0) continue;
            const int32_t at = s[r].crow.x + (int32_t)(rnd[r].x % (uint32_t)deg);
            // (evict-first in L2 where the adjacency dwarfs it: DevGraph::adj_streams)
            if (fat) {
                const int4 f = g.adj_streams ? ld_once(g.fat + at) : __ldg(g.fat + at);
                nxt[r] = f.x;
                nrow[r] = make_int2(f.y, f.z);
            } else {
                nxt[r] = g.adj_streams ? ld_once(g.adj + at) : __ldg(g.adj + at);
            }
            moved[r] = true;
        }
    } else if (S == kAlias) {
        // static_alias_interleaving_move (alias_sampling.h:221-258)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (s[r].widx < 0) continue;
            const int32_t deg = s[r].crow.y - s[r].crow.x;
            if (deg > 0) {
                const AliasSlot a = load_alias(g.alias + s[r].crow.x + (int32_t)(rnd[r].x % (uint32_t)deg));
                nxt[r] = real2_le(rnd[r].y, a.prob) ? a.first : a.second;
                moved[r] = true;
            }
        }
    } else if (S == kITS) {
        // static_its_interleaving_move (inverse_transformation_sampling.h:36-145):
        // target = real2 * P[last], then the branchless upper bound of
        // utility.h:18-27 advanced one probe per ring slot per round.
        double t[R];
        const double *base[R];
        int32_t n[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            n[r] = 0;
            if (s[r].widx < 0) continue;
            const int32_t deg = s[r].crow.y - s[r].crow.x;
            if (deg <= 0) continue;
            const double total = __ldg(g.prefix + s[r].crow.y - 1);
            if (total == 0.0) continue;  // zero-weight row: the walker stops
            t[r] = real2(rnd[r].x) * total;
            base[r] = g.prefix + s[r].crow.x;
            n[r] = deg;
        }
        bool more = true;
        while (more) {
            more = false;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (n[r] > 1) {
                    const int32_t half = n[r] >> 1;
                    base[r] = (__ldg(base[r] + half) <= t[r]) ? base[r] + half : base[r];
                    n[r] -= half;
                    more |= n[r] > 1;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (n[r] == 1) {
                const int32_t sel = (int32_t)((__ldg(base[r]) <= t[r]) + (base[r] - (g.prefix + s[r].crow.x)));
                nxt[r] = __ldg(g.adj + s[r].crow.x + sel);
                moved[r] = true;
            }
        }
    } else if (S == kLabelIndex) {
        // MetaPath's dynamic ITS over its 0/1 label weights (metapath.cpp:22-30,
        // inverse_transformation_sampling.h:288-313): the upper bound over the
        // 0/1 prefix sums picks match floor(count * real2) of the wanted label
        // in row order, which the label index holds at lab_nbr[off[l] + m]
        // (an empty row or a label without match: the walker stops).
        int32_t lo[R], cnt[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            cnt[r] = 0;
            if (s[r].widx < 0) continue;
            if (fat) {  // the block came with the entry of the last move (or at admission)
                lo[r] = s[r].crow.x;
                cnt[r] = s[r].crow.y - s[r].crow.x;
                continue;
            }
            const int32_t want = p.schema[(s[r].len - 1) % p.schema_len];
            if (want < 0 || want >= g.lab_k) continue;  // a label no edge has: no match
            const int32_t *off = g.lab_off + (int64_t)s[r].cur * (g.lab_k + 1) + want;
            lo[r] = __ldg(off);
            cnt[r] = __ldg(off + 1) - lo[r];
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (cnt[r] <= 0) continue;
            const int32_t m = (int32_t)((double)cnt[r] * real2(rnd[r].x));  // floor of P[last] * dr_
            if (fat) {
                const int4 f = __ldg(g.lab_fat + lo[r] + m);
                nxt[r] = f.x;
                nrow[r] = make_int2(f.y, f.z);
            } else {
                nxt[r] = __ldg(g.lab_nbr + lo[r] + m);
            }
            moved[r] = true;
        }
    } else if (S == kRejection) {
        // static_rs_move (rejection_sampling.h:334-366): trial k uses draws 2k, 2k+1.
        double mx[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (s[r].widx >= 0) mx[r] = __ldg(g.rmax + s[r].cur);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (s[r].widx < 0) continue;
            const int32_t deg = s[r].crow.y - s[r].crow.x;
            if (deg <= 0) continue;
            DrawCursor c(p.seed, (uint64_t)(p.id_base + s[r].widx), (uint32_t)s[r].len, rnd[r]);
            uint32_t trials = 0;
            int32_t p0;
            for (;;) {
                p0 = (int32_t)(c.next() % (uint32_t)deg);
                const double y = real2(c.next()) * mx[r];
                const double w = p.static_unit ? 1.0 : __ldg(g.weight + s[r].crow.x + p0);
                if (y <= w) break;
                if (++trials >= kMaxTrials) break;
            }
            if (trials >= kMaxTrials) { atomicOr(p.error, kErrTrials); continue; }
            nxt[r] = __ldg(g.adj + s[r].crow.x + p0);
            moved[r] = true;
        }
    } else {
        // dynamic max-weight rejection: dr_ = max_weight (creeper.h:648-653), then
        // per trial position, app weight, real2 * max (rejection_sampling.h:368-402).
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (s[r].widx < 0) continue;
            const int32_t deg = s[r].crow.y - s[r].crow.x;
            if (deg <= 0) continue;
            DrawCursor c(p.seed, (uint64_t)(p.id_base + s[r].widx), (uint32_t)s[r].len, rnd[r]);
            uint32_t trials = 0;
            int32_t nb;
            int2 nbrow = make_int2(0, 0);
            for (;;) {
                const int32_t p0 = (int32_t)(c.next() % (uint32_t)deg);
                if (fat) {
                    const int4 f = __ldg(g.fat + s[r].crow.x + p0);
                    nb = f.x;
                    nbrow = make_int2(f.y, f.z);
                } else {
                    nb = __ldg(g.adj + s[r].crow.x + p0);
                }
                bool accept;
                if (WK == kNode2Vec) {
                    accept = n2v_accept(p, s[r].len, s[r].prev, s[r].prow, nb, c.next());
                } else if (WK == kUnitWeight) {
                    accept = c.next() <= p.accept_max[2];
                } else {
                    const double w = app_weight<WK>(p, s[r].len, s[r].prev, s[r].prow, nb, s[r].crow.x + p0);
                    accept = real2(c.next()) * p.max_weight <= w;
                }
                if (accept) break;
                if (++trials >= kMaxTrials) break;
            }
            if (trials >= kMaxTrials) { atomicOr(p.error, kErrTrials); continue; }
            nxt[r] = nb;
            nrow[r] = nbrow;
            moved[r] = true;
        }
    }

    // Move bookkeeping (e.g. alias_sampling.h:251-255) and update
    // (creeper.h:299-319).
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (s[r].widx < 0) continue;
        if (!moved[r]) { finish<path_gather<S>(), R>(p, s[r], r); continue; }
        s[r].prev = s[r].cur;
        if (S != kLabelIndex) s[r].prow = s[r].crow;  // (the label index reads no row pair)
        s[r].cur = nxt[r];
        if (fat) s[r].crow = nrow[r];
        if (p.paths && s[r].len < p.path_cap) path_put<path_gather<S>(), R>(p, s[r], r, s[r].len, nxt[r]);
        s[r].len += 1;
        steps += 1;
        if (kSparse) {
            const unsigned peers = __match_any_sync(__activemask(), ((unsigned long long)s[r].q << 32) | (uint32_t)nxt[r]);
            if ((threadIdx.x & 31) == __ffs(peers) - 1) start_insert(p, pend[r][0], s[r].q, nxt[r], __popc(peers));
        } else {
            record_visit(p, s[r].q, nxt[r]);
        }
        if (app_update<U>(p, (uint64_t)(p.id_base + s[r].widx), s[r].len)) finish<path_gather<S>(), R>(p, s[r], r);
    }
}

__device__ __forceinline__ void flush_steps(const WalkParams &p, uint64_t steps) {
    unsigned long long v = steps;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(p.steps, v);
}

template <int S, int U, int WK, int R, bool kSparse>
__global__ void __launch_bounds__(kThreadBlock) walk_persistent(const WalkParams p) {
    const int lane = threadIdx.x & 31;
    constexpr unsigned long long kChunk = 32ull * R * 2;
    Slot s[R];
    PendingInsert pend[R][kInsertDepth];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        s[r].widx = -1;
#pragma unroll
        for (int k = 0; k < kInsertDepth; ++k) pend[r][k].q = -1;
    }
    uint64_t steps = 0;
    unsigned long long res_next = 0, res_end = 0;
    bool drained = false;
    for (;;) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            unsigned need = __ballot_sync(kFull, s[r].widx < 0);
            while (need && !drained) {
                if (res_next >= res_end) {
                    unsigned long long b = 0;
                    if (lane == 0) b = atomicAdd(p.queue_head, kChunk);
                    b = __shfl_sync(kFull, b, 0);
                    if (b >= (unsigned long long)p.num_walkers) { drained = true; break; }
                    res_next = b;
                    res_end = min(b + kChunk, (unsigned long long)p.num_walkers);
                }
                const unsigned avail = (unsigned)min(res_end - res_next, 32ull);
                const unsigned rank = __popc(need & lanemask_lt());
                const bool mine = ((need >> lane) & 1u) && rank < avail;
                if (mine) admit<S, R>(p, s[r], r, (int64_t)(res_next + rank));
                res_next += min((unsigned)__popc(need), avail);
                need &= ~__ballot_sync(kFull, mine);
            }
        }
        bool live = false;
#pragma unroll
        for (int r = 0; r < R; ++r) live |= s[r].widx >= 0;
        if (!__any_sync(kFull, live)) break;
        step_ring<S, U, WK, R, kSparse>(p, s, steps, pend);
    }
    if (kSparse) {
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int k = 0; k < kInsertDepth; ++k) resolve(p, pend[r][k], true);
    }
    flush_steps(p, steps);
}

template <int S, int U, int WK, bool kSparse>
__global__ void __launch_bounds__(kThreadBlock) walk_plain(const WalkParams p) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t steps = 0;
    if (idx < p.num_walkers) {
        Slot s[1];
        PendingInsert pend[1][kInsertDepth];
            for (int k = 0; k < kInsertDepth; ++k) pend[0][k].q = -1;
        admit<S, 1>(p, s[0], 0, idx);
        while (s[0].widx >= 0) step_ring<S, U, WK, 1, kSparse>(p, s, steps, pend);
        if (kSparse)
            for (int k = 0; k < kInsertDepth; ++k) resolve(p, pend[0][k], true);
    }
    flush_steps(p, steps);
}

// Multi-request form of the persistent engine (ring depth 1, the serving
// loop's batches): a warp claims chunks of kMultiChunk walkers of one request
// from the shared queue (the admission of creeper.h:321-332 over many
// requests' walkers), and each lane steps its walker with its own request's
// parameters (read through L1 from the request table).  PPR requests record
// each move in their own table, lanes of the warp on the same (request,
// vertex) merged first; each finished walker adds its moves to its
// request's step counter, and the lane that finishes a request's last walker
// raises the request's completion flag in host memory.
template <int S, int U, int WK>
__global__ void __launch_bounds__(kThreadBlock) walk_multi(const MultiBatch mb, const int64_t total_chunks) {
    const int lane = threadIdx.x & 31;
    Slot s[1];
    s[0].widx = -1;
    PendingInsert pend[1][kInsertDepth];
    pend[0][0].q = -1;
    int32_t req = 0;      // this lane's walker's request
    uint32_t wsteps = 0;  // its moves so far
    int32_t r_req = 0;    // the warp's current chunk: request, next walker, end
    int64_t r_next = 0, r_end = 0;
    bool drained = false;
    for (;;) {
        unsigned need = __ballot_sync(kFull, s[0].widx < 0);
        while (need && !drained) {
            if (r_next >= r_end) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(mb.queue_head, 1ull);
                b = __shfl_sync(kFull, b, 0);
                if (b >= (unsigned long long)total_chunks) { drained = true; break; }
                int32_t lo = 0, hi = mb.nreq;  // request r with chunk_start[r] <= b < chunk_start[r + 1]
                while (hi - lo > 1) {
                    const int32_t mid = (lo + hi) >> 1;
                    if (__ldg(mb.chunk_start + mid) <= (int64_t)b) lo = mid; else hi = mid;
                }
                r_req = lo;
                r_next = ((int64_t)b - __ldg(mb.chunk_start + lo)) * kMultiChunk;
                r_end = min(r_next + kMultiChunk, mb.reqs[lo].num_walkers);
            }
            const unsigned avail = (unsigned)min(r_end - r_next, (int64_t)32);
            const unsigned rank = __popc(need & lanemask_lt());
            const bool mine = ((need >> lane) & 1u) && rank < avail;
            bool dead = false;
            if (mine) {
                req = r_req;
                wsteps = 0;
                admit<S, 1>(mb.reqs[req], s[0], 0, r_next + rank);
                dead = s[0].widx < 0;  // an invalid source finishes at once
            }
            if (dead) {
                __threadfence();
                const unsigned peers = __match_any_sync(__activemask(), req);
                if (lane == __ffs(peers) - 1) {
                    const int n = __popc(peers);
                    if (atomicSub(mb.remaining + req, n) == n && mb.done[req]) {
                        __threadfence_system();
                        *mb.done[req] = 1;
                    }
                }
            }
            r_next += min((unsigned)__popc(need), avail);
            need &= ~__ballot_sync(kFull, mine);
        }
        if (!__any_sync(kFull, s[0].widx >= 0)) break;
        const WalkParams &p = mb.reqs[req];
        const bool was = s[0].widx >= 0;
        const int32_t len0 = s[0].len;
        uint64_t moved = 0;
        step_ring<S, U, WK, 1, false>(p, s, moved, pend);
        wsteps += (uint32_t)moved;
        if (mb.tables && was && s[0].len != len0) {  // a PPR move to s[0].cur
            int32_t *t = mb.tables[req];
            if (t) {
                const unsigned peers =
                    __match_any_sync(__activemask(), ((unsigned long long)(uint32_t)req << 32) | (uint32_t)s[0].cur);
                if (lane == __ffs(peers) - 1) table_add(t, mb.table_bits[req], s[0].cur, __popc(peers), mb.error);
            }
        }
        if (was && s[0].widx < 0) {  // the walker finished
            const unsigned peers = __match_any_sync(__activemask(), req);
            const unsigned total = __reduce_add_sync(peers, wsteps);
            __threadfence();  // this group's outputs and moves before the countdown
            if (lane == __ffs(peers) - 1) {
                atomicAdd(p.steps, (unsigned long long)total);
                __threadfence();
                const int n = __popc(peers);
                if (atomicSub(mb.remaining + req, n) == n && mb.done[req]) {
                    __threadfence_system();
                    *mb.done[req] = 1;
                }
            }
        }
    }
}

template <class K>
int max_occupancy(K kernel) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kThreadBlock, 0) != cudaSuccess || n <= 0) n = 1;
    return n;
}

template <int S, int U, int WK, int R, bool kSparse>
cudaError_t launch_persistent(const WalkParams &p, const LaunchShape &shape, cudaStream_t st) {
    static const int max_occ = max_occupancy(walk_persistent<S, U, WK, R, kSparse>);
    const int per_sm = shape.ctas_per_sm > 0 ? min(shape.ctas_per_sm, max_occ) : max_occ;
    int64_t grid = (int64_t)shape.num_sms * per_sm;
    const int64_t useful = (p.num_walkers + (int64_t)kThreadBlock * R - 1) / ((int64_t)kThreadBlock * R);
    if (useful < grid) grid = useful;
    if (grid <= 0) return cudaSuccess;
    walk_persistent<S, U, WK, R, kSparse><<<(unsigned)grid, kThreadBlock, 0, st>>>(p);
    return cudaGetLastError();
}

template <int S, int U, int WK, bool kSparse>
cudaError_t launch_mode(const WalkParams &p, const LaunchShape &shape, cudaStream_t st) {
    if (shape.engine == kEnginePlain) {
        const int64_t blocks = (p.num_walkers + kThreadBlock - 1) / kThreadBlock;
        if (blocks <= 0) return cudaSuccess;
        walk_plain<S, U, WK, kSparse><<<(unsigned)blocks, kThreadBlock, 0, st>>>(p);
        return cudaGetLastError();
    }
    switch (shape.ring) {
    case 1: return launch_persistent<S, U, WK, 1, kSparse>(p, shape, st);
    case 2: return launch_persistent<S, U, WK, 2, kSparse>(p, shape, st);
    case 8: return launch_persistent<S, U, WK, 8, kSparse>(p, shape, st);
    default: return launch_persistent<S, U, WK, 4, kSparse>(p, shape, st);
    }
}

// Sparse visit tables only exist for PPR (geometric update).
template <int S, int U, int WK>
cudaError_t launch_shape(const WalkParams &p, const LaunchShape &shape, cudaStream_t st) {
    if constexpr (U == kGeometric) {
        if (p.table) return launch_mode<S, U, WK, true>(p, shape, st);
    }
    return launch_mode<S, U, WK, false>(p, shape, st);
}

template <int S, int U, int WK>
cudaError_t launch_multi(const MultiBatch &mb, int64_t total_walkers, int64_t total_chunks, int num_sms,
                         cudaStream_t st) {
    static const int max_occ = max_occupancy(walk_multi<S, U, WK>);
    int64_t grid = (int64_t)num_sms * max_occ;
    const int64_t useful = (total_walkers + kThreadBlock - 1) / kThreadBlock;
    if (useful < grid) grid = useful;
    if (grid <= 0 || mb.nreq <= 0 || total_chunks <= 0) return cudaSuccess;
    walk_multi<S, U, WK><<<(unsigned)grid, kThreadBlock, 0, st>>>(mb, total_chunks);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_walk_multi(const MultiBatch &mb, int64_t total_walkers, int64_t total_chunks, int sampler,
                              int update, int weight_kind, int num_sms, cudaStream_t st) {
    const bool geo = update == kGeometric;
    switch (sampler) {
    case kUniform: return geo ? launch_multi<kUniform, kGeometric, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st)
                              : launch_multi<kUniform, kFixedLength, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st);
    case kAlias: return geo ? launch_multi<kAlias, kGeometric, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st)
                            : launch_multi<kAlias, kFixedLength, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st);
    case kITS: return geo ? launch_multi<kITS, kGeometric, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st)
                          : launch_multi<kITS, kFixedLength, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st);
    case kRejection:
        return geo ? launch_multi<kRejection, kGeometric, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st)
                   : launch_multi<kRejection, kFixedLength, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st);
    case kLabelIndex: return launch_multi<kLabelIndex, kFixedLength, kLabelSchema>(mb, total_walkers, total_chunks, num_sms, st);
    case kMaxRejection:
        if (weight_kind == kNode2Vec)
            return launch_multi<kMaxRejection, kFixedLength, kNode2Vec>(mb, total_walkers, total_chunks, num_sms, st);
        if (weight_kind == kEdgeWeight)
            return launch_multi<kMaxRejection, kFixedLength, kEdgeWeight>(mb, total_walkers, total_chunks, num_sms, st);
        if (geo) return launch_multi<kMaxRejection, kGeometric, kUnitWeight>(mb, total_walkers, total_chunks, num_sms, st);
        return cudaErrorInvalidValue;
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_walk_thread(const WalkParams &p, int sampler, int update, int weight_kind,
                               const LaunchShape &shape, cudaStream_t st) {
    const bool geo = update == kGeometric;
    switch (sampler) {
    case kUniform: return geo ? launch_shape<kUniform, kGeometric, kUnitWeight>(p, shape, st)
                              : launch_shape<kUniform, kFixedLength, kUnitWeight>(p, shape, st);
    case kAlias: return geo ? launch_shape<kAlias, kGeometric, kUnitWeight>(p, shape, st)
                            : launch_shape<kAlias, kFixedLength, kUnitWeight>(p, shape, st);
    case kITS: return geo ? launch_shape<kITS, kGeometric, kUnitWeight>(p, shape, st)
                          : launch_shape<kITS, kFixedLength, kUnitWeight>(p, shape, st);
    case kRejection: return geo ? launch_shape<kRejection, kGeometric, kUnitWeight>(p, shape, st)
                                : launch_shape<kRejection, kFixedLength, kUnitWeight>(p, shape, st);
    case kLabelIndex: return launch_shape<kLabelIndex, kFixedLength, kLabelSchema>(p, shape, st);
    case kMaxRejection:
        if (weight_kind == kNode2Vec) return launch_shape<kMaxRejection, kFixedLength, kNode2Vec>(p, shape, st);
        if (weight_kind == kEdgeWeight) return launch_shape<kMaxRejection, kFixedLength, kEdgeWeight>(p, shape, st);
        if (geo) return launch_shape<kMaxRejection, kGeometric, kUnitWeight>(p, shape, st);
        return cudaErrorInvalidValue;
    }
    return cudaErrorInvalidValue;
}

}  // namespace trw
