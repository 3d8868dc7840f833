// trw_ppr_sparse.cu -- sparse per-query PPR visit counts.
//
// During the walk every move adds the new vertex to its query's
// open-addressing table (table_add, trw_device.cuh).  Walker ids are claimed
// in increasing order, so only the tables of the few dozen queries whose
// walkers are in flight are being written at any time and they stay in L2;
// the dense query-major alternative (4 x N bytes per query) would need its
// whole count array zeroed every batch.
//
// After the walk:
//  * distinct_kernel + segment_scan_kernel + offsets_kernel: occupied slots
//    per warp segment of each table, their prefix within the query, then the
//    queries' totals scanned into CSR offsets (offsets[q] .. offsets[q+1] hold query
//    q's entries), continuing from offsets[0] so that a batch can run as
//    several ranges of queries;
//  * emit_kernel (one CTA per chunk of at most 2^16 slots): writes the
//    (vertex, count) pairs.  With
//    linear probing the SET of occupied slots does not depend on the order of
//    insertion, only the order of keys inside each run of occupied slots
//    does; so the kernel emits runs in slot order (the run that wraps around
//    the table end last) with the keys inside each run sorted, which makes
//    the output a function of the visit counts alone.  It then zeroes the
//    table for the next batch.
#include "trw_device.cuh"
#include "trw_internal.h"

namespace trw {
namespace {

constexpr int kScanThreads = 256;
constexpr int kEmitThreads = 256;

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

constexpr int kEmitWarps = kEmitThreads / 32;  // table segments per CTA

// A table of 2^bits slots is split into chunks_for(bits, cbits) chunks of at
// most 2^cbits slots (2^16 by default), one CTA each, and every chunk into
// kEmitWarps warp segments; a single large table (a query with many walkers)
// is then spread over the GPU instead of one CTA.  Smaller chunks shorten a
// CTA's run where few tables fill the GPU (the ranges of a host-output batch).
__host__ __device__ inline uint32_t chunks_for(int32_t bits, int32_t cbits) {
    return bits > cbits ? 1u << (bits - cbits) : 1u;
}

// Occupied slots (distinct visited vertices) per warp segment: seg[(q * S +
// chunk) * kEmitWarps + warp].
__global__ void __launch_bounds__(kEmitThreads) distinct_kernel(const int32_t *tables, int32_t bits, int32_t cbits,
                                                                 int32_t *seg) {
    const uint32_t S = chunks_for(bits, cbits);
    const int64_t q = blockIdx.x / S;
    const uint32_t c = blockIdx.x % S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t chunk = (1u << bits) / S;
    const uint32_t seg4 = chunk / kEmitWarps / 4;  // int4 per segment
    const int4 *keys = reinterpret_cast<const int4 *>(tables + (q << (bits + 1)) + (size_t)c * chunk) + warp * seg4;
    uint32_t n = 0;
    for (uint32_t i = lane; i < seg4; i += 32) {
        const int4 k = __ldg(keys + i);
        n += (k.x != 0) + (k.y != 0) + (k.z != 0) + (k.w != 0);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if (lane == 0) seg[((int64_t)blockIdx.x) * kEmitWarps + warp] = (int32_t)n;
}

// Per query: the segment counts become their exclusive prefix within the
// query (in place) and the query's total goes to distinct[q].
__global__ void __launch_bounds__(kScanThreads) segment_scan_kernel(int32_t *seg, int32_t bits, int32_t cbits,
                                                                     int32_t *distinct) {
    __shared__ int32_t sums[32];
    const int64_t q = blockIdx.x;
    const int32_t n = (int32_t)chunks_for(bits, cbits) * kEmitWarps;
    int32_t *v = seg + q * n;
    int32_t carry = 0;
    for (int32_t b = 0; b < n; b += kScanThreads) {
        const int32_t i = b + threadIdx.x;
        const int32_t x = i < n ? v[i] : 0;
        int32_t total;
        const int32_t ex = block_exclusive_scan<int32_t>(x, sums, total);
        if (i < n) v[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) distinct[q] = carry;
}

// offsets[0] holds the entries of the queries before this range (0 for the
// first range of a batch); offsets[1..nq] become the running totals.
__global__ void __launch_bounds__(kScanThreads) offsets_kernel(const int32_t *distinct, int64_t nq, int64_t *offsets) {
    __shared__ int64_t sums[32];
    int64_t carry = offsets[0];  // read by every thread before the first write below
    for (int64_t b = 0; b < nq; b += kScanThreads) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < nq ? (int64_t)distinct[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan<int64_t>(v, sums, total);
        if (i < nq) offsets[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) offsets[nq] = carry;
}

// One CTA per chunk of at most 2^cbits slots of a query's table, one contiguous
// segment of the chunk per warp.
//
// Output order.  Inserts probe linearly and wrap from the last slot to slot
// 0, so the occupied slots form maximal runs on a cycle; which slots are
// occupied, and which keys each run holds, do not depend on the order of the
// inserts, only the order of the keys inside a run does.  The entries are
// written run by run in slot order, each run's keys sorted, except that the
// run wrapping around the table end (if any) comes last.  Each occupied slot
// finds its own output position:
//   pos = (occupied slots before it) - (slots of the wrapping run at the table
//         start) - (its distance back to the run start) + (rank of its key
//         among the run's keys)
// A warp takes 128 slots of its segment per iteration (segments are
// multiples of 128 slots: tables have at least 2^10 slots, chunks 2^10 to
// 2^16, 8 warps a CTA).  Counts arrive two blocks ahead into a per-warp
// buffer of the current block.  Keys arrive with 16-byte loads into a per-warp ring
// of four 128-slot blocks in shared memory (the previous, current and next
// block, and the one after being filled); four ballots per block give its
// 128-bit occupancy.  The block's occupied slots are dealt out to the lanes
// in order (lane l takes occupied slots l, l + 32, ..., located with
// find-nth-set-bit in the occupancy words), so every lane has a slot to emit
// instead of 58 % of them idling on empty ones.  Each slot finds the empty
// slots before and after its run with clz/ffs in its own 32-slot word and the
// neighbouring ones, and ranks its key by reading the run from the ring.  Runs reaching further (rare at the
// tables' load) and the run that wraps around the table end are read from
// global memory, which stays intact until the zeroing.  (Searching the whole
// 384-slot window instead cost 5 % more post-processing time on GB300.)
constexpr int32_t kBlk4 = 128;
constexpr int32_t kRing = 4 * kBlk4;

__global__ void __launch_bounds__(kEmitThreads) emit_kernel(int32_t *tables, int32_t bits, int32_t cbits,
                                                             const int64_t *offsets, const int32_t *seg_prefix,
                                                             int32_t *vout, int32_t *cout, int64_t capacity,
                                                             int *error) {
    __shared__ uint32_t wrap[2];
    __shared__ __align__(16) int32_t ring_all[kEmitWarps][kRing];
    __shared__ uint32_t wsm_all[kEmitWarps][6];  // occupancy words 3 .. 8 of the window
    __shared__ __align__(16) int32_t cnt_all[kEmitWarps][kBlk4];  // counts of the current block
    const uint32_t S = chunks_for(bits, cbits);
    const int64_t q = blockIdx.x / S;
    const uint32_t chunk = blockIdx.x % S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nslots = 1u << bits;
    int32_t *keys = tables + (q << (bits + 1));
    const int32_t *cnts = keys + nslots;
    const int4 *k4 = reinterpret_cast<const int4 *>(keys);
    const int64_t end = offsets[q + 1];
    const bool write = end <= capacity;
    if (threadIdx.x == 0) {
        if (!write && chunk == 0) atomicOr(error, kErrCapacity);
        uint32_t head = 0, tail = 0;
        if (__ldg(keys) != 0 && __ldg(keys + nslots - 1) != 0) {
            while (head < nslots && __ldg(keys + head) != 0) ++head;
            if (head < nslots) {
                while (__ldg(keys + nslots - 1 - tail) != 0) ++tail;
            } else {
                head = 0;  // a full table (the walk reported it) has no run boundary
            }
        }
        wrap[0] = head;
        wrap[1] = tail;
    }
    __syncthreads();
    const uint32_t head = wrap[0], tail = wrap[1], cyc = head + tail;
    int64_t prefix = offsets[q] + seg_prefix[(int64_t)blockIdx.x * kEmitWarps + warp];
    const uint32_t seg = nslots / S / kEmitWarps;  // a multiple of kBlk4 here
    const uint32_t lo = chunk * (nslots / S) + warp * seg;
    const int32_t nblk = (int32_t)(seg / kBlk4);
    int32_t *ring = ring_all[warp];
    // block m (slots lo + 128 m ...) sits at ring[((m + 1) * 128) mod 512 ...]
    auto load_blk = [&](int32_t m) {
        const int64_t y0 = (int64_t)lo + (int64_t)m * kBlk4;
        return y0 >= 0 && y0 < (int64_t)nslots ? __ldg(k4 + (y0 >> 2) + lane) : make_int4(0, 0, 0, 0);
    };
    auto ring_of = [&](int32_t m) { return ring + (((m + 1) * kBlk4) & (kRing - 1)); };
    auto ballots = [&](int32_t m, uint32_t(&o)[4]) {
        const int32_t *r = ring_of(m);
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = __ballot_sync(0xffffffffu, r[32 * j + lane] != 0);
    };
    reinterpret_cast<int4 *>(ring_of(-1))[lane] = load_blk(-1);
    reinterpret_cast<int4 *>(ring_of(0))[lane] = load_blk(0);
    reinterpret_cast<int4 *>(ring_of(1))[lane] = load_blk(1);
    int4 kf = load_blk(2);
    // counts of block m (16 bytes a lane), loaded two blocks ahead so that no
    // iteration waits on a DRAM round trip for them
    const int4 *c4 = reinterpret_cast<const int4 *>(cnts);
    auto load_cnt = [&](int32_t m) {
        return m < nblk ? __ldg(c4 + (((int64_t)lo + (int64_t)m * kBlk4) >> 2) + lane) : make_int4(0, 0, 0, 0);
    };
    int4 ca = load_cnt(0), cb = load_cnt(1);
    int32_t *cbuf = cnt_all[warp];
    uint32_t *wsm = wsm_all[warp];
    __syncwarp();
    uint32_t w[12];  // occupancy of the window: blocks b - 1, b, b + 1, 32 slots a word
    {
        uint32_t o[4];
        ballots(-1, o);
#pragma unroll
        for (int j = 0; j < 4; ++j) w[j] = o[j];
        ballots(0, o);
#pragma unroll
        for (int j = 0; j < 4; ++j) w[4 + j] = o[j];
        ballots(1, o);
#pragma unroll
        for (int j = 0; j < 4; ++j) w[8 + j] = o[j];
    }
    for (int32_t b = 0; b < nblk; ++b) {
        reinterpret_cast<int4 *>(ring_of(b + 2))[lane] = kf;  // over block b - 2, read before the last __syncwarp
        kf = load_blk(b + 3);
        reinterpret_cast<int4 *>(cbuf)[lane] = ca;  // over block b - 1's, read before the last __syncwarp
        ca = cb;
        cb = load_cnt(b + 2);
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) wsm[i] = w[3 + i];
        }
        __syncwarp();
        // the block's occupied slots, compacted: lane l takes occupied slots
        // l, l + 32, ... of the block (m counts the occupied slots before it)
        const uint32_t c1 = __popc(w[4]), c2 = c1 + __popc(w[5]), c3 = c2 + __popc(w[6]), n = c3 + __popc(w[7]);
        for (uint32_t m0 = 0; m0 < n; m0 += 32) {
            const uint32_t m = m0 + lane;
            if (!write || m >= n) continue;
            int wi;
            uint32_t rem;
            if (m < c1) { wi = 0; rem = m; }
            else if (m < c2) { wi = 1; rem = m - c1; }
            else if (m < c3) { wi = 2; rem = m - c2; }
            else { wi = 3; rem = m - c3; }
            const uint32_t wc = wsm[wi + 1];
            const int bit = (int)__fns(wc, 0, (int)rem + 1);
            const int32_t p = kBlk4 + 32 * wi + bit;  // this slot's window position
            const uint32_t xs = lo + (uint32_t)b * kBlk4 + 32 * wi + bit;
            const int32_t k = ring[(b * kBlk4 + p) & (kRing - 1)];
            int64_t pos;
            if (cyc && (xs < head || xs + tail >= nslots)) {  // the wrap-around run: last, keys sorted
                uint32_t rank = 0;
                for (uint32_t i = 0; i < cyc; ++i) {
                    const uint32_t y = i < tail ? nslots - tail + i : i - tail;
                    rank += __ldg(keys + y) < k;
                }
                pos = end - cyc + rank;
            } else {
                // the empty window positions before (s) and after (e) the run,
                // from this word and its neighbours (runs reaching further take
                // the global path below)
                int32_t s = -1, e = 3 * kBlk4;
                uint32_t z = ~wc & ((1u << bit) - 1u);
                if (z) {
                    s = 32 * (4 + wi) + 31 - __clz(z);
                } else {
                    const uint32_t wp = wsm[wi];
                    if (~wp) s = 32 * (3 + wi) + 31 - __clz(~wp);
                }
                z = ~wc & ~((2u << bit) - 1u);
                if (z) {
                    e = 32 * (4 + wi) + __ffs(z) - 1;
                } else {
                    const uint32_t wn = wsm[wi + 2];
                    if (~wn) e = 32 * (5 + wi) + __ffs(~wn) - 1;
                }
                uint32_t rank = 0, back;
                if (s >= 0 && e < 3 * kBlk4) {
                    back = (uint32_t)(p - s - 1);
                    for (int32_t i = s + 1; i < e; ++i)
                        rank += ring[(b * kBlk4 + i) & (kRing - 1)] < k;  // k itself does not count
                } else {  // the run reaches beyond the window
                    back = 0;
                    while (xs > back && __ldg(keys + xs - back - 1) != 0) ++back;
                    for (uint32_t d = 1; d <= back; ++d) rank += __ldg(keys + xs - d) < k;
                    for (uint32_t y = xs + 1; y < nslots; ++y) {
                        const int32_t v = __ldg(keys + y);
                        if (v == 0) break;
                        rank += v < k;
                    }
                }
                pos = prefix + m - head - back + rank;
            }
            vout[pos] = k - 1;
            cout[pos] = cbuf[32 * wi + bit] + 1;  // the table counts visits after the first
        }
        prefix += n;
        __syncwarp();
        uint32_t o[4];
        ballots(b + 2, o);
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = w[j + 4];
#pragma unroll
        for (int j = 0; j < 4; ++j) w[8 + j] = o[j];
    }
    if (S > 1) return;  // chunked tables are zeroed after the kernel: other CTAs may still read this chunk
    __syncthreads();
    int4 *zr = reinterpret_cast<int4 *>(keys);
    for (uint32_t i = threadIdx.x; i < nslots / 2; i += blockDim.x) zr[i] = make_int4(0, 0, 0, 0);
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

int64_t ppr_distinct_ints(int32_t bits, int32_t chunk_bits) {
    return 1 + (int64_t)chunks_for(bits, chunk_bits) * kEmitWarps;
}

cudaError_t launch_ppr_offsets(const int32_t *tables, int32_t bits, int32_t *distinct, int64_t nq, int64_t *offsets,
                               cudaStream_t st, int32_t chunk_bits) {
    if (nq > 0) {
        const int64_t ctas = nq * chunks_for(bits, chunk_bits);
        distinct_kernel<<<(unsigned)ctas, kEmitThreads, 0, st>>>(tables, bits, chunk_bits, distinct + nq);
        segment_scan_kernel<<<(unsigned)nq, kScanThreads, 0, st>>>(distinct + nq, bits, chunk_bits, distinct);
    }
    offsets_kernel<<<1, kScanThreads, 0, st>>>(distinct, nq, offsets);
    return cudaGetLastError();
}

cudaError_t launch_ppr_emit(int32_t *tables, int32_t bits, int64_t nq, const int64_t *offsets,
                            const int32_t *distinct, int32_t *vout, int32_t *cout, int64_t capacity, int *error,
                            cudaStream_t st, int32_t chunk_bits) {
    if (nq <= 0) return cudaSuccess;
    const uint32_t S = chunks_for(bits, chunk_bits);
    emit_kernel<<<(unsigned)(nq * S), kEmitThreads, 0, st>>>(tables, bits, chunk_bits, offsets, distinct + nq, vout,
                                                             cout, capacity, error);
    if (S > 1) return cudaMemsetAsync(tables, 0, sizeof(int32_t) * 2 * ((size_t)nq << bits), st);
    return cudaGetLastError();
}

}  // namespace trw
