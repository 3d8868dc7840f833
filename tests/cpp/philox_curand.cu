// TEST PROGRAM: the engine's device Philox4x32-10 (draw_block in
// thunderrw_gb300/csrc/trw_device.cuh, written from Salmon et al., SC'11)
// against cuRAND's Philox4_32_10 generator run on the same key and counter.
// The engine's counter for (walker, step, block) is the 128-bit value
// block | step << 32 | walker << 64 under key = seed; cuRAND's state after
// curand_init(seed, subsequence = walker, offset = 4 * (block | step << 32))
// sits on that counter, so its next curand4() must give the same four words.
#include <cstdio>
#include <cstdint>
#include <curand_kernel.h>

#include "trw_device.cuh"

__global__ void draw_both(int n, uint4 *ours, uint4 *theirs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t seeds[4] = {1ull, 0x123456789ABCDEF0ull, 0xFFFFFFFFFFFFFFFFull, 20240601ull};
    const uint64_t seed = seeds[i & 3];
    const uint64_t walker = (uint64_t)i * 2654435761ull + ((uint64_t)(i % 7) << 40);
    const uint32_t step = (uint32_t)i * 7u + 1u;
    const uint32_t block = (i % 5 == 0) ? trw::kTermBlock : (uint32_t)(i % 3);
    ours[i] = trw::draw_block(seed, walker, step, block);
    curandStatePhilox4_32_10_t st;
    curand_init(seed, walker, ((uint64_t)step << 32 | block) * 4ull, &st);
    theirs[i] = curand4(&st);
}

int main() {
    const int n = 1 << 16;
    uint4 *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(uint4) * n) != cudaSuccess) { std::printf("cudaMalloc failed\n"); return 2; }
    draw_both<<<(n + 255) / 256, 256>>>(n, d, d + n);
    static uint4 h[2 << 16];
    if (cudaMemcpy(h, d, 2 * sizeof(uint4) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
        std::printf("kernel or copy failed\n");
        return 2;
    }
    int bad = 0;
    for (int i = 0; i < n; ++i) {
        const uint4 a = h[i], b = h[n + i];
        if (a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w) {
            if (bad < 4) std::printf("mismatch %d: %08x %08x %08x %08x vs %08x %08x %08x %08x\n", i, a.x, a.y, a.z,
                                     a.w, b.x, b.y, b.z, b.w);
            ++bad;
        }
    }
    std::printf("%d of %d blocks differ\n", bad, n);
    cudaFree(d);
    return bad ? 1 : 0;
}
