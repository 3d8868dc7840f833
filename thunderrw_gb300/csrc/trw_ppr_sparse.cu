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
//  * distinct_kernel + offsets_kernel: occupied slots per query, then their
//    exclusive scan into CSR offsets (offsets[q] .. offsets[q+1] hold query
//    q's entries);
//  * emit_kernel (one CTA per query): writes the (vertex, count) pairs.  With
//    linear probing the SET of occupied slots does not depend on the order of
//    insertion, only the order of keys inside each run of occupied slots
//    does; so the kernel emits slots in order with the keys inside each run
//    sorted, which makes the output a function of the visit counts alone.
//    It then zeroes the table for the next batch.
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

constexpr int kEmitWarps = kEmitThreads / 32;  // table segments per query

// Occupied slots (distinct visited vertices) of each query's table, per
// segment of 1/kEmitWarps of the slots (the emit kernel's warp split) and in
// total.
__global__ void __launch_bounds__(kEmitThreads) distinct_kernel(const int32_t *tables, int32_t bits, int32_t *distinct,
                                                                int32_t *seg_counts) {
    const int64_t q = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t seg4 = (1u << bits) / kEmitWarps / 4;  // int4 per segment
    const int4 *keys = reinterpret_cast<const int4 *>(tables + (q << (bits + 1))) + warp * seg4;
    uint32_t c = 0;
    for (uint32_t i = lane; i < seg4; i += 32) {
        const int4 k = __ldg(keys + i);
        c += (k.x != 0) + (k.y != 0) + (k.z != 0) + (k.w != 0);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ uint32_t ws[kEmitWarps];
    if (lane == 0) { ws[warp] = c; seg_counts[q * kEmitWarps + warp] = (int32_t)c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kEmitWarps; ++w) t += ws[w];
        distinct[q] = (int32_t)t;
    }
}

__global__ void __launch_bounds__(kScanThreads) offsets_kernel(const int32_t *distinct, int64_t nq, int64_t *offsets) {
    __shared__ int64_t sums[32];
    int64_t carry = 0;
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

constexpr uint32_t kRing = 8;   // staged 32-slot blocks per warp
constexpr uint32_t kAhead = 3;  // blocks staged ahead of the one being emitted

// One CTA per query, one contiguous segment of the table per warp.  Output
// order: slots in index order, the keys of each run of occupied slots sorted
// (runs end at the end of the table).  Which slots are occupied does not
// depend on the insertion order, so this order depends on the counts alone.
// Every occupied slot finds its own output position:
//   pos = (occupied slots before it) - (its distance back to the run start)
//         + (rank of its key among the run's keys)
// A warp walks its segment 32 slots at a time with coalesced loads, keeping a
// ring of staged blocks in shared memory so that run neighbours within one
// block behind and kAhead blocks ahead are read from there; farther ones
// (rare) come from global memory, which stays intact until the final zeroing.
__global__ void __launch_bounds__(kEmitThreads) emit_kernel(int32_t *tables, int32_t bits, const int64_t *offsets,
                                                            const int32_t *seg_counts, int32_t *vout, int32_t *cout,
                                                            int64_t capacity, int *error) {
    __shared__ int32_t ring[kEmitWarps][kRing * 32];
    __shared__ int32_t cring[kEmitWarps][kRing * 32];
    const int64_t q = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nslots = 1u << bits;
    int32_t *keys = tables + (q << (bits + 1));
    int32_t *cnts = keys + nslots;
    const bool write = offsets[q + 1] <= capacity;
    if (!write && threadIdx.x == 0) atomicOr(error, kErrCapacity);
    int64_t prefix = offsets[q];
    for (int w = 0; w < warp; ++w) prefix += seg_counts[q * kEmitWarps + w];

    const uint32_t seg = nslots / kEmitWarps;  // >= 64: tables have >= 1024 slots
    const uint32_t lo = warp * seg, nblk = seg / 32;
    int32_t *rk = ring[warp];
    int32_t *rc = cring[warp];
    // block j of the segment lives in ring slot j % kRing, block -1 in the last slot
    auto stage = [&](uint32_t j) {
        const uint32_t x = lo + j * 32 + lane;
        const int k = x < nslots ? __ldg(keys + x) : 0;
        rk[(j % kRing) * 32 + lane] = k;
        rc[(j % kRing) * 32 + lane] = k ? __ldg(cnts + x) : 0;
    };
    rk[(kRing - 1) * 32 + lane] = lo ? __ldg(keys + lo - 32 + lane) : 0;
    for (uint32_t j = 0; j < kAhead; ++j) stage(j);
    for (uint32_t b = 0; b < nblk; ++b) {
        const uint32_t x0 = lo + b * 32, x = x0 + lane;
        stage(b + kAhead);
        __syncwarp();
        const int key = rk[(b % kRing) * 32 + lane];
        const unsigned occm = __ballot_sync(0xffffffffu, key != 0);
        const int64_t before = prefix + __popc(occm & ((1u << lane) - 1u));
        prefix += __popc(occm);
        if (write && key != 0) {
            const uint32_t slo = x0 >= 32 ? x0 - 32 : 0, shi = x0 + (kAhead + 1) * 32;
            auto nkey = [&](uint32_t y) {
                if (y >= slo && y < shi) return rk[((y - lo) / 32 % kRing) * 32 + (y & 31)];
                return y < nslots ? __ldg(keys + y) : 0;
            };
            uint32_t back = 0;
            while (x > back && nkey(x - back - 1) != 0) ++back;
            uint32_t rank = 0;
            for (uint32_t d = 1; d <= back; ++d) rank += nkey(x - d) < key;
            for (uint32_t y = x + 1; y < nslots; ++y) {
                const int k2 = nkey(y);
                if (k2 == 0) break;
                rank += k2 < key;
            }
            const int64_t pos = before - back + rank;
            vout[pos] = key - 1;
            cout[pos] = rc[(b % kRing) * 32 + lane];
        }
        __syncwarp();
    }
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kEmitWarps; ++w) t += seg_counts[q * kEmitWarps + w];
        if (t != offsets[q + 1] - offsets[q]) atomicOr(error, kErrCapacity);
    }
    __syncthreads();
    // zero the table for the next batch (coalesced 16-byte stores)
    int4 *z = reinterpret_cast<int4 *>(keys);
    for (uint32_t i = threadIdx.x; i < nslots / 2; i += blockDim.x) z[i] = make_int4(0, 0, 0, 0);
}

}  // namespace

cudaError_t launch_ppr_offsets(const int32_t *tables, int32_t bits, int32_t *distinct, int64_t nq, int64_t *offsets,
                               cudaStream_t st) {
    if (nq > 0) distinct_kernel<<<(unsigned)nq, kEmitThreads, 0, st>>>(tables, bits, distinct, distinct + nq);
    offsets_kernel<<<1, kScanThreads, 0, st>>>(distinct, nq, offsets);
    return cudaGetLastError();
}

cudaError_t launch_ppr_emit(int32_t *tables, int32_t bits, int64_t nq, const int64_t *offsets,
                            const int32_t *distinct, int32_t *vout, int32_t *cout, int64_t capacity, int *error,
                            cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    emit_kernel<<<(unsigned)nq, kEmitThreads, 0, st>>>(tables, bits, offsets, distinct + nq, vout, cout, capacity,
                                                       error);
    return cudaGetLastError();
}

}  // namespace trw
