// Throughput probe of the visibility raster's depth test: 64-bit
// reductions `red.relaxed.gpu.global.max.u64` (write_fragment in
// lh_device.cuh) over a buffer, with no return value, as fast as the grid
// can issue them.  The reductions per second it reaches are the roofline
// denominator of the raster's fragment traffic: a raster whose fragments
// approach it is bound by the L2 atomic units, one far below it by
// something else (instruction issue, load latency).  No counterpart in the
// reference (its depth test is fixed-function).
#include <cuda_runtime.h>

#include <cstdint>

#include "lh/lh.h"

namespace lh {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    // splitmix64 finaliser: a fixed bijection of the word index, so
    // `scattered` reductions land on pseudo-random words of the buffer
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return x;
}

// reps passes over the n words; pass r sends key (r << 32 | i) to word i
// (contiguous: a warp covers 256 consecutive bytes, as the chunk raster's
// rows do) or to word mix64(i + r * n) mod n (scattered: every lane its own
// line, as the lane raster's small triangles do).
__global__ void __launch_bounds__(256) k_probe_red_u64(unsigned long long* words, uint64_t n, uint32_t scattered,
                                                      uint32_t reps) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint32_t r = 0; r < reps; r++)
        for (uint64_t i = tid; i < n; i += stride) {
            const uint64_t w = scattered ? mix64(i + (uint64_t)r * n) % n : i;
            const unsigned long long key = ((unsigned long long)r << 32) | (uint32_t)i;
            asm volatile("red.relaxed.gpu.global.max.u64 [%0], %1;" ::"l"(words + w), "l"(key) : "memory");
        }
}

}  // namespace
}  // namespace lh

extern "C" lh_status lh_probe_red_u64(uint64_t* d_words, uint64_t n_words, uint32_t scattered, uint32_t reps,
                                      void* stream) {
    if (!d_words || ((uintptr_t)d_words & 7) || n_words == 0 || reps == 0) return LH_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return LH_ERR_CUDA;
    const uint64_t want = (n_words + 255) / 256;
    const unsigned blocks = (unsigned)(want < (uint64_t)sms * 8 ? want : (uint64_t)sms * 8);
    lh::k_probe_red_u64<<<blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<unsigned long long*>(d_words), n_words, scattered ? 1u : 0u, reps);
    return cudaGetLastError() == cudaSuccess ? LH_OK : LH_ERR_CUDA;
}
