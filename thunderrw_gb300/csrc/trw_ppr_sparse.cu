// trw_ppr_sparse.cu -- sparse per-query PPR visit counts: the post-processing
// kernel that turns a batch's visits into CSR (offsets, vertex, count).
//
// Each query's counts live in an open-addressing table of 2^bits slots (key
// vertex + 1, 0 = empty), cut into sub-tables of 2^sb slots, sb =
// sub_bits(bits) <= 13; a vertex's sub-table is the top bits of its home slot
// and linear probing wraps around inside the sub-table (trw_device.cuh).  A
// sub-table fits one CTA's shared memory (64 KB at sb = 13, three CTAs per
// SM), so one CTA handles one (query, sub-table) tile:
//  * build the sub-table in shared memory, either from the query's visit
//    logs (the persistent engine's log form: the walk appended every move to
//    its item's segment for the vertex's sub-table, so the tile reads only its
//    own segments) or from the table the walk filled in global memory (table
//    form: plain engine, very large queries), which it then zeroes;
//  * count its occupied slots and find the tile's output offset by a
//    decoupled look-back over the tiles before it (tiles are claimed in
//    order from a counter, so every tile it waits for is running);
//  * write its entries: the runs of occupied slots in slot order with the
//    keys of each run sorted, the run that wraps around the sub-table's end
//    last.  Which slots are occupied and which keys each run holds do not
//    depend on the order of the inserts, so the output is a function of the
//    counts (and the table geometry) alone.
// Tiles go in (query, sub-table) order, so a query's entries are contiguous.
#include "trw_device.cuh"
#include "trw_internal.h"

namespace trw {
namespace {

constexpr int kPostThreads = 512;  // three CTAs (tiles) per SM at sb = 13
constexpr unsigned long long kFlagAgg = 1ull << 62;   // tile count published
constexpr unsigned long long kFlagPref = 1ull << 63;  // tile's inclusive offset published
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr uint32_t kLookbackSpins = 1u << 17;  // per window of predecessors, ~100 ns each

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *warp_sums, T &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    total = warp_sums[nw - 1];
    const T before = warp ? warp_sums[warp - 1] : T(0);
    const T excl = before + x - v;
    __syncthreads();
    return excl;
}

// Adds one visit of v (if `mine`) to the shared-memory sub-table; lanes with
// the same vertex are merged first (a query's walkers revisit the vertices
// around its source).
__device__ __forceinline__ void smem_add(int32_t *keys, int32_t *cnts, uint32_t M, uint32_t home, int32_t v,
                                         bool mine, int *error) {
    if (!mine) return;
    const unsigned peers = __match_any_sync(__activemask(), v);
    if ((int)(threadIdx.x & 31) != __ffs(peers) - 1) return;
    const int inc = __popc(peers);
    const int32_t key = v + 1;
    volatile int32_t *vk = keys;
    uint32_t h = home & (M - 1u);
    for (uint32_t probe = 0; probe < M; ++probe) {
        int32_t k = vk[h];
        if (k == 0) k = atomicCAS(keys + h, 0, key);
        if (k == 0 || k == key) {
            atomicAdd(cnts + h, inc);
            return;
        }
        h = (h + 1u) & (M - 1u);
    }
    atomicOr(error, kErrCapacity);  // the sub-table is full
}

__global__ void __launch_bounds__(kPostThreads, 3) ppr_post_kernel(const PprPost pp) {
    extern __shared__ __align__(16) int32_t sm[];
    __shared__ long long s_tile, s_excl;
    __shared__ uint32_t s_head, s_tail;
    __shared__ int32_t s_sums[32];
    const int32_t sb = sub_bits(pp.bits);
    const uint32_t M = 1u << sb, W = M >> 5;  // bits >= 10: W >= 32 words
    const int32_t pbits = pp.bits - sb;        // sub-tables per query: 2^pbits
    int32_t *keys = sm, *cnts = sm + M;
    uint32_t *words = reinterpret_cast<uint32_t *>(sm + 2 * M);
    int32_t *wpre = reinterpret_cast<int32_t *>(words + W);
    int32_t *ipre = wpre + W;  // log form: prefix of the query's item segment lengths
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;

    if (tid == 0) s_tile = (long long)atomicAdd(pp.tile_next, 1u);
    int4 *sm4 = reinterpret_cast<int4 *>(sm);
    for (uint32_t i = tid; i < M / 2; i += blockDim.x) sm4[i] = make_int4(0, 0, 0, 0);
    __syncthreads();
    const int64_t tile = s_tile;
    const int64_t q = tile >> pbits;
    const uint32_t sub = (uint32_t)(tile & ((1ll << pbits) - 1));

    // ---- build the sub-table
    if (pp.tables) {
        // the walk's global table: counts hold visits minus one; zero it for the next batch
        int4 *tk = reinterpret_cast<int4 *>(pp.tables + (q << (pp.bits + 1)) + ((int64_t)sub << sb));
        int4 *tc = reinterpret_cast<int4 *>(pp.tables + (q << (pp.bits + 1)) + (1ll << pp.bits) + ((int64_t)sub << sb));
        int4 *k4 = sm4, *c4 = reinterpret_cast<int4 *>(cnts);
        for (uint32_t i = tid; i < M / 4; i += blockDim.x) {
            const int4 k = __ldcg(tk + i), c = __ldcg(tc + i);
            k4[i] = k;
            c4[i] = make_int4(k.x ? c.x + 1 : 0, k.y ? c.y + 1 : 0, k.z ? c.z + 1 : 0, k.w ? c.w + 1 : 0);
            tk[i] = make_int4(0, 0, 0, 0);
            tc[i] = make_int4(0, 0, 0, 0);
        }
    } else {
        // This tile's segment of each of the query's item logs: a prefix over
        // their lengths in shared memory, then one flattened loop in which
        // every thread loads four entries before inserting them.
        const int32_t ipq = pp.items_per_query;  // <= kLogMaxItems
        const int64_t seg0 = (q * ipq << pbits) + sub;  // segment of the query's first item
        int32_t carry = 0;
        for (int32_t b = 0; b < ipq; b += blockDim.x) {
            const int32_t i = b + tid;
            const int32_t n = i < ipq ? __ldcg(pp.log_fill + seg0 + ((int64_t)i << pbits)) : 0;
            int32_t tot;
            const int32_t ex = block_exclusive_scan<int32_t>(n, s_sums, tot);
            if (i < ipq) ipre[i] = carry + ex;
            carry += tot;
        }
        if (tid == 0) ipre[ipq] = carry;
        __syncthreads();
        const int32_t entries = carry;
        for (int32_t e0 = 0; e0 < entries; e0 += 4 * (int32_t)blockDim.x) {
            int32_t v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int32_t e = e0 + u * (int32_t)blockDim.x + tid;
                v[u] = -1;
                if (e < entries) {
                    int32_t lo = 0, hi = ipq;  // item i with ipre[i] <= e < ipre[i + 1]
                    while (hi - lo > 1) {
                        const int32_t mid = (lo + hi) >> 1;
                        if (ipre[mid] <= e) lo = mid; else hi = mid;
                    }
                    v[u] = __ldcg(pp.log + (seg0 + ((int64_t)lo << pbits)) * pp.log_seg + (e - ipre[lo]));
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t home = v[u] >= 0 ? ppr_home(v[u], pp.bits) : 0u;
                smem_add(keys, cnts, M, home, v[u], v[u] >= 0, pp.error);
            }
        }
        // the query's overflow entries (rare), those of this sub-table
        const int32_t no = min(__ldcg(pp.log_ovf_n + q), pp.log_ovf_cap);
        for (int32_t j = tid; j < no; j += blockDim.x) {
            const int32_t v = __ldcg(pp.log_ovf + q * pp.log_ovf_cap + j);
            const uint32_t home = ppr_home(v, pp.bits);
            smem_add(keys, cnts, M, home, v, (home >> sb) == sub, pp.error);
        }
    }
    __syncthreads();

    // ---- occupancy words, their prefix counts and the wrap-around run
    for (uint32_t w = warp; w < W; w += nwarps) {
        const unsigned b = __ballot_sync(0xffffffffu, keys[w * 32 + lane] != 0);
        if (lane == 0) words[w] = b;
    }
    __syncthreads();
    int32_t total;
    const int32_t pc = tid < (int)W ? __popc(words[tid]) : 0;  // W <= 256 < blockDim
    const int32_t pex = block_exclusive_scan<int32_t>(pc, s_sums, total);
    if (tid < (int)W) wpre[tid] = pex;
    if (tid == 0) {
        uint32_t head = 0, tail = 0;
        if ((words[0] & 1u) && (words[W - 1] >> 31) && total < (int32_t)M) {
            for (uint32_t w = 0;; ++w) {
                const uint32_t inv = ~words[w];
                if (inv) { head += __ffs(inv) - 1; break; }
                head += 32;
            }
            for (uint32_t w = W - 1;; --w) {
                const uint32_t inv = ~words[w];
                if (inv) { tail += __clz(inv); break; }
                tail += 32;
            }
        }
        s_head = head;
        s_tail = tail;
    }

    // ---- the tile's output offset: decoupled look-back by warp 0, over 32
    // predecessors per round trip (lane i examines tile j - i)
    if (warp == 0) {
        int64_t excl = 0;
        if (tile == 0) {
            excl = pp.offsets[0];
        } else {
            if (lane == 0) atomicExch(pp.status + tile, kFlagAgg | (unsigned long long)total);
            int64_t j = tile - 1;
            uint32_t spins = 0;
            for (;;) {
                const int64_t idx = j - lane;
                // before the first tile: a neutral prefix of 0 (tile 0 always publishes one)
                const unsigned long long w = idx >= 0 ? *reinterpret_cast<volatile unsigned long long *>(pp.status + idx)
                                                      : (unsigned long long)kFlagPref;
                const unsigned pref = __ballot_sync(0xffffffffu, (w & kFlagPref) != 0);
                const unsigned any = __ballot_sync(0xffffffffu, (w & (kFlagPref | kFlagAgg)) != 0);
                int take = -1;  // lanes 0..take are summed
                if (pref) {
                    const int f = __ffs(pref) - 1;  // the nearest inclusive prefix
                    const unsigned nearer = (1u << f) - 1u;
                    if ((any & nearer) == nearer) take = f;
                } else if (any == 0xffffffffu) {
                    take = 31;
                }
                if (take >= 0) {
                    unsigned long long v = lane <= take ? (w & kValMask) : 0ull;
#pragma unroll
                    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    excl += (int64_t)v;
                    if (pref) break;
                    j -= 32;
                    spins = 0;
                    continue;
                }
                if (++spins > kLookbackSpins) {  // a nearer tile has not published (cannot happen)
                    if (lane == 0) atomicOr(pp.error, kErrLookback);
                    break;
                }
                __nanosleep(100);
            }
        }
        if (lane == 0) {
            atomicExch(pp.status + tile, kFlagPref | (unsigned long long)(excl + total));
            s_excl = excl;
            if (sub == 0) pp.offsets[q] = excl;
            if (tile == (pp.nq << pbits) - 1) pp.offsets[pp.nq] = excl + total;
            if (excl + total > pp.capacity) atomicOr(pp.error, kErrCapacity);
        }
    }
    __syncthreads();

    // ---- entries in canonical order
    const int64_t excl = s_excl;
    if (excl + total > pp.capacity) return;
    const uint32_t head = s_head, tail = s_tail, cyc = head + tail;
    for (uint32_t x = tid; x < M; x += blockDim.x) {
        const int32_t k = keys[x];
        if (k == 0) continue;
        int32_t pos;
        if (x < head || x + tail >= M) {  // the wrap-around run: last, keys sorted
            uint32_t rank = 0;
            for (uint32_t i = 0; i < cyc; ++i) {
                const uint32_t y = i < tail ? M - tail + i : i - tail;
                rank += keys[y] < k;
            }
            pos = total - (int32_t)cyc + (int32_t)rank;
        } else {
            uint32_t back = 0;
            while (x > back && keys[x - back - 1] != 0) ++back;
            uint32_t rank = 0;
            for (uint32_t d = 1; d <= back; ++d) rank += keys[x - d] < k;
            for (uint32_t y = x + 1; y < M && keys[y] != 0; ++y) rank += keys[y] < k;
            const uint32_t before = (uint32_t)wpre[x >> 5] + __popc(words[x >> 5] & ((1u << (x & 31)) - 1u));
            pos = (int32_t)(before - head - back + rank);
        }
        pp.vout[excl + pos] = k - 1;
        pp.cout[excl + pos] = cnts[x];
    }
}

__global__ void sum_steps_kernel(const unsigned long long *parts, int n, unsigned long long *out) {
    unsigned long long t = 0;
    for (int i = 0; i < n; ++i) t += parts[i];
    *out = t;
}

}  // namespace

cudaError_t launch_sum_steps(const uint64_t *parts, int n, uint64_t *out, cudaStream_t st) {
    sum_steps_kernel<<<1, 1, 0, st>>>(reinterpret_cast<const unsigned long long *>(parts), n,
                                      reinterpret_cast<unsigned long long *>(out));
    return cudaGetLastError();
}

size_t ppr_post_smem(int32_t bits) {
    const size_t M = (size_t)1 << sub_bits(bits);
    return 2 * M * sizeof(int32_t) + 2 * (M / 32) * sizeof(int32_t) + (kLogMaxItems + 1) * sizeof(int32_t);
}

cudaError_t launch_ppr_post(const PprPost &pp, cudaStream_t st) {
    if (pp.nq <= 0) return cudaSuccess;
    static const cudaError_t attr = cudaFuncSetAttribute(ppr_post_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)ppr_post_smem(30));
    if (attr != cudaSuccess) return attr;
    const int64_t tiles = pp.nq << (pp.bits - sub_bits(pp.bits));
    ppr_post_kernel<<<(unsigned)tiles, kPostThreads, ppr_post_smem(pp.bits), st>>>(pp);
    return cudaGetLastError();
}

}  // namespace trw
