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

constexpr int kScanThreads = 1024;
constexpr int kEmitThreads = 512;

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
constexpr int32_t kChunkBits = 16;             // at most 2^16 slots per CTA

// A table of 2^bits slots is split into chunks_for(bits) chunks of at most
// 2^16 slots, one CTA each, and every chunk into kEmitWarps warp segments;
// a single large table (a query with many walkers) is then spread over the
// GPU instead of one CTA.
__host__ __device__ inline uint32_t chunks_for(int32_t bits) {
    return bits > kChunkBits ? 1u << (bits - kChunkBits) : 1u;
}

// Occupied slots (distinct visited vertices) per warp segment: seg[(q * S +
// chunk) * kEmitWarps + warp].
__global__ void __launch_bounds__(kEmitThreads) distinct_kernel(const int32_t *tables, int32_t bits, int32_t *seg) {
    const uint32_t S = chunks_for(bits);
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
__global__ void __launch_bounds__(kScanThreads) segment_scan_kernel(int32_t *seg, int32_t bits, int32_t *distinct) {
    __shared__ int32_t sums[32];
    const int64_t q = blockIdx.x;
    const int32_t n = (int32_t)chunks_for(bits) * kEmitWarps;
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

// One CTA per chunk of at most 2^16 slots of a query's table, one contiguous
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
// A warp walks its segment 32 slots at a time with coalesced loads and keeps
// the previous, current and next blocks of keys in registers (two more blocks
// in flight): the run of a slot is found from the three occupancy ballots and
// its key ranked against the run through shuffles.  Runs reaching beyond that
// 96-slot window, and the wrapping run, are read from global memory, which
// stays intact until the final zeroing.
__global__ void __launch_bounds__(kEmitThreads) emit_kernel(int32_t *tables, int32_t bits, const int64_t *offsets,
                                                            const int32_t *seg_prefix, int32_t *vout, int32_t *cout,
                                                            int64_t capacity, int *error) {
    __shared__ uint32_t wrap[2];
    const uint32_t S = chunks_for(bits);
    const int64_t q = blockIdx.x / S;
    const uint32_t chunk = blockIdx.x % S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nslots = 1u << bits;
    int32_t *keys = tables + (q << (bits + 1));
    int32_t *cnts = keys + nslots;
    const int64_t end = offsets[q + 1];
    const bool write = end <= capacity;
    if (threadIdx.x == 0) {
        if (!write && chunk == 0) atomicOr(error, kErrCapacity);
        // the wrapping run: `head` slots from slot 0 and `tail` slots before the end
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

    const uint32_t seg = nslots / S / kEmitWarps;  // >= 64: tables have >= 1024 slots, chunks 2^16
    const uint32_t lo = chunk * (nslots / S) + warp * seg, nblk = seg / 32;
    const uint32_t x0 = lo + lane;
    auto key_at = [&](uint32_t y) { return y < nslots ? __ldg(keys + y) : 0; };
    auto cnt_at = [&](uint32_t y) { return y < nslots ? __ldg(cnts + y) : 0; };
    int32_t kp = lo ? __ldg(keys + lo - 32 + lane) : 0;
    int32_t kc = key_at(x0), cc = cnt_at(x0);
    int32_t kn = key_at(x0 + 32), cn = cnt_at(x0 + 32);
    int32_t k2 = key_at(x0 + 64), c2 = cnt_at(x0 + 64);
    unsigned op = __ballot_sync(0xffffffffu, kp != 0);
    const unsigned lt = lanemask_lt(), le = lt | (1u << lane);
    for (uint32_t b = 0; b < nblk; ++b) {
        const uint32_t x = x0 + b * 32;
        const int32_t k3 = key_at(x + 96), c3 = cnt_at(x + 96);
        const unsigned oc = __ballot_sync(0xffffffffu, kc != 0), on = __ballot_sync(0xffffffffu, kn != 0);
        const int64_t before = prefix + __popc(oc & lt);
        prefix += __popc(oc);
        const bool in_wrap = kc != 0 && (x < head || x >= nslots - tail);
        // window positions: 0-31 previous block, 32-63 this block, 64-95 next block
        int s = -1, e = -1;
        if (kc != 0 && !in_wrap) {
            const unsigned zb = ~oc & lt, za = ~oc & ~le;
            if (zb) s = 64 - __clz(zb);
            else if (~op) s = 32 - __clz(~op);
            if (za) e = 31 + __ffs(za);
            else if (~on) e = 63 + __ffs(~on);
        }
        const bool fast = s >= 0 && e >= 0;
        const int len = fast ? e - s : 0;
        const int maxlen = __reduce_max_sync(0xffffffffu, len);
        uint32_t rank = 0;
        if (__all_sync(0xffffffffu, !fast || (s >= 32 && e <= 64))) {
            // every run of this block lies inside it: rank within this block's keys
            for (int d = 0; d < maxlen; ++d) {
                const int j = s + d;
                const int32_t k = __shfl_sync(0xffffffffu, kc, j & 31);
                if (d < len && j != 32 + lane) rank += k < kc;
            }
        } else {
            for (int d = 0; d < maxlen; ++d) {
                const int j = s + d;
                const int src = j & 31;
                const int32_t a = __shfl_sync(0xffffffffu, kp, src);
                const int32_t m = __shfl_sync(0xffffffffu, kc, src);
                const int32_t n = __shfl_sync(0xffffffffu, kn, src);
                const int32_t k = j < 32 ? a : j < 64 ? m : n;
                if (d < len && j != 32 + lane) rank += k < kc;
            }
        }
        if (write && kc != 0) {
            int64_t pos;
            if (fast) {
                pos = before - head - (32 + lane - s) + rank;
            } else if (in_wrap) {
                rank = 0;
                for (uint32_t i = 0; i < cyc; ++i) {
                    const uint32_t y = i < tail ? nslots - tail + i : i - tail;
                    rank += __ldg(keys + y) < kc;
                }
                pos = end - cyc + rank;
            } else {
                uint32_t back = 0;
                while (x > back && __ldg(keys + x - back - 1) != 0) ++back;
                rank = 0;
                for (uint32_t d = 1; d <= back; ++d) rank += __ldg(keys + x - d) < kc;
                for (uint32_t y = x + 1; y < nslots; ++y) {
                    const int32_t k = __ldg(keys + y);
                    if (k == 0) break;
                    rank += k < kc;
                }
                pos = before - head - back + rank;
            }
            vout[pos] = kc - 1;
            cout[pos] = cc + 1;  // the table counts visits after the first
        }
        kp = kc; op = oc;
        kc = kn; cc = cn;
        kn = k2; cn = c2;
        k2 = k3; c2 = c3;
    }
    if (S > 1) return;  // chunked tables are zeroed after the kernel: other CTAs may still read this chunk
    __syncthreads();
    // zero the table for the next batch (coalesced 16-byte stores)
    int4 *z = reinterpret_cast<int4 *>(keys);
    for (uint32_t i = threadIdx.x; i < nslots / 2; i += blockDim.x) z[i] = make_int4(0, 0, 0, 0);
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

int64_t ppr_distinct_ints(int32_t bits) { return 1 + (int64_t)chunks_for(bits) * kEmitWarps; }

cudaError_t launch_ppr_offsets(const int32_t *tables, int32_t bits, int32_t *distinct, int64_t nq, int64_t *offsets,
                               cudaStream_t st) {
    if (nq > 0) {
        const int64_t ctas = nq * chunks_for(bits);
        distinct_kernel<<<(unsigned)ctas, kEmitThreads, 0, st>>>(tables, bits, distinct + nq);
        segment_scan_kernel<<<(unsigned)nq, kScanThreads, 0, st>>>(distinct + nq, bits, distinct);
    }
    offsets_kernel<<<1, kScanThreads, 0, st>>>(distinct, nq, offsets);
    return cudaGetLastError();
}

cudaError_t launch_ppr_emit(int32_t *tables, int32_t bits, int64_t nq, const int64_t *offsets,
                            const int32_t *distinct, int32_t *vout, int32_t *cout, int64_t capacity, int *error,
                            cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    const uint32_t S = chunks_for(bits);
    emit_kernel<<<(unsigned)(nq * S), kEmitThreads, 0, st>>>(tables, bits, offsets, distinct + nq, vout, cout,
                                                             capacity, error);
    if (S > 1) return cudaMemsetAsync(tables, 0, sizeof(int32_t) * 2 * ((size_t)nq << bits), st);
    return cudaGetLastError();
}

}  // namespace trw
