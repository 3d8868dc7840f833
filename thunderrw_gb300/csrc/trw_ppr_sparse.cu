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
//    does; so the kernel emits runs in slot order (from the first empty
//    slot) with the keys inside each run sorted, which makes the output a
//    function of the visit counts alone.  It then zeroes the table for the
//    next batch.
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

// Number of occupied slots (distinct visited vertices) of each query's table.
__global__ void __launch_bounds__(kScanThreads) distinct_kernel(const int32_t *tables, int32_t bits, int32_t *distinct) {
    __shared__ uint32_t sums[32];
    const int64_t q = blockIdx.x;
    const int4 *keys = reinterpret_cast<const int4 *>(tables + (q << (bits + 1)));
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < (1u << bits) / 4; i += blockDim.x) {
        const int4 k = __ldg(keys + i);
        c += (k.x != 0) + (k.y != 0) + (k.z != 0) + (k.w != 0);
    }
    uint32_t total;
    block_exclusive_scan<uint32_t>(c, sums, total);
    if (threadIdx.x == 0) distinct[q] = (int32_t)total;
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

constexpr uint32_t kChunkSlots = 2048;  // table slots staged in shared memory per round
constexpr uint32_t kPer = kChunkSlots / kEmitThreads;

// One CTA per query.  Output order: the table's slots in order starting just
// after its first empty slot e (so no run of occupied slots wraps around),
// each run's keys sorted.  Every occupied slot finds its own output position:
//   pos = (occupied slots before its run's first slot) + (rank of its key in the run)
// where, because a run is contiguous, the first term is the occupied-slot
// prefix at the slot minus its distance to the run start.  The table is
// staged chunk by chunk in shared memory; zeroing lags one chunk so that runs
// crossing a chunk boundary can still be read from the previous chunk.
__global__ void __launch_bounds__(kEmitThreads) emit_kernel(int32_t *tables, int32_t bits, const int64_t *offsets,
                                                            int32_t *vout, int32_t *cout, int64_t capacity,
                                                            int *error) {
    __shared__ int32_t sk[kChunkSlots];
    __shared__ int32_t sc[kChunkSlots];
    __shared__ uint32_t sums[32];
    __shared__ uint32_t s_first_empty;
    const int64_t q = blockIdx.x;
    const uint32_t nslots = 1u << bits, mask = nslots - 1u;
    int32_t *keys = tables + (q << (bits + 1));
    int32_t *cnts = keys + nslots;
    const uint32_t cn = min(kChunkSlots, nslots);
    const uint32_t per = cn / blockDim.x;
    const int64_t base = offsets[q];
    const bool write = offsets[q + 1] <= capacity;
    if (!write && threadIdx.x == 0) atomicOr(error, kErrCapacity);

    // first empty slot (a table holding fewer keys than slots always has one)
    if (threadIdx.x < 32) {
        uint32_t e = mask;
        bool found = false;
        for (uint32_t b = 0; b < nslots; b += 32) {
            const unsigned m = __ballot_sync(0xffffffffu, __ldg(keys + b + threadIdx.x) == 0);
            if (m) { e = b + __ffs(m) - 1; found = true; break; }
        }
        if (threadIdx.x == 0) {
            s_first_empty = e;
            if (!found) atomicOr(error, kErrCapacity);  // a full table has no run boundary
        }
    }
    __syncthreads();
    const uint32_t start = (s_first_empty + 1) & mask;  // logical index 0
    auto slot = [&](uint32_t logical) { return (start + logical) & mask; };

    int64_t done = 0;  // occupied slots before the current chunk
    for (uint32_t c0 = 0; c0 < nslots; c0 += cn) {
        for (uint32_t i = threadIdx.x; i < cn; i += blockDim.x) {
            const uint32_t j = slot(c0 + i);
            sk[i] = __ldg(keys + j);
            sc[i] = __ldg(cnts + j);
        }
        __syncthreads();
        const uint32_t lo = threadIdx.x * per;
        uint32_t mine = 0;
        for (uint32_t k = 0; k < per; ++k) mine += sk[lo + k] != 0;
        uint32_t total;
        const uint32_t excl = block_exclusive_scan<uint32_t>(mine, sums, total);
        if (write) {
            int64_t prefix = done + excl;  // occupied slots before logical c0 + lo + k
            for (uint32_t k = 0; k < per; ++k) {
                const uint32_t i = lo + k;
                const int key = sk[i];
                if (key == 0) continue;
                // distance back to the run's first slot (the previous chunk is still intact)
                uint32_t back = 0;
                while (true) {
                    const uint32_t li = c0 + i - back;  // logical index of the slot examined
                    if (li == 0) break;                 // logical 0 follows an empty slot
                    const int pk = (i >= back + 1) ? sk[i - back - 1] : __ldg(keys + slot(li - 1));
                    if (pk == 0) break;
                    if (++back >= cn) { atomicOr(error, kErrCapacity); break; }  // run longer than a chunk
                }
                // rank of the key among the run's keys
                uint32_t rank = 0;
                for (uint32_t d = 1; d <= back; ++d) {
                    const int pk = (i >= d) ? sk[i - d] : __ldg(keys + slot(c0 + i - d));
                    rank += pk < key;
                }
                for (uint32_t d = 1; c0 + i + d < nslots; ++d) {
                    const int nk = (i + d < cn) ? sk[i + d] : __ldg(keys + slot(c0 + i + d));
                    if (nk == 0) break;
                    rank += nk < key;
                }
                const int64_t pos = base + prefix - back + rank;
                vout[pos] = key - 1;
                cout[pos] = sc[i];
                ++prefix;
            }
        }
        done += total;
        __syncthreads();
        if (c0 != 0) {  // zero the previous chunk: no run of this chunk reaches further back
            for (uint32_t i = threadIdx.x; i < cn; i += blockDim.x) {
                const uint32_t j = slot(c0 - cn + i);
                keys[j] = 0;
                cnts[j] = 0;
            }
        }
    }
    for (uint32_t i = threadIdx.x; i < cn; i += blockDim.x) {
        const uint32_t j = slot(nslots - cn + i);
        keys[j] = 0;
        cnts[j] = 0;
    }
    if (threadIdx.x == 0 && done != offsets[q + 1] - base) atomicOr(error, kErrCapacity);
}

}  // namespace

cudaError_t launch_ppr_offsets(const int32_t *tables, int32_t bits, int32_t *distinct, int64_t nq, int64_t *offsets,
                               cudaStream_t st) {
    if (nq > 0) distinct_kernel<<<(unsigned)nq, kScanThreads, 0, st>>>(tables, bits, distinct);
    offsets_kernel<<<1, kScanThreads, 0, st>>>(distinct, nq, offsets);
    return cudaGetLastError();
}

cudaError_t launch_ppr_emit(int32_t *tables, int32_t bits, int64_t nq, const int64_t *offsets, int32_t *vout,
                            int32_t *cout, int64_t capacity, int *error, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    emit_kernel<<<(unsigned)nq, kEmitThreads, 0, st>>>(tables, bits, offsets, vout, cout, capacity, error);
    return cudaGetLastError();
}

}  // namespace trw
