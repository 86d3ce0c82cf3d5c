// Instance cull + single-pass prefix sum that allocates nothing.
//
// Some callers cannot call cudaMalloc: an engine that owns every byte of
// device memory under a fixed budget and forbids hidden allocations, a frame
// loop that must never stall (cudaMalloc can synchronise the whole device),
// or code that records work while a stream is being captured.  This entry
// point serves them: the caller passes the scene and the output sector, and
// the only scratch the kernel needs -- the look-back words of its tiles and
// the tile claim counter -- lives in a fixed array compiled into this library
// (`g_cull_scratch` below, about 33 KB, held by every GPU that loads the
// library until the process exits).
//
// Limits and rules of use:
//  - at most kNoAllocMaxTiles tiles of kInstTile instances (1,048,576
//    instances); larger calls are rejected with LH_ERR_CAPACITY;
//  - a call made outside stream capture looks up the device address of the
//    array (cudaGetSymbolAddress) with the caller's device current and keeps
//    it for that device; a call made while its stream is being captured uses
//    the address kept by the last call outside capture, so make the first
//    call on a device before any stream capture (after a cudaDeviceReset,
//    or under another context, make one call outside capture again);
//  - every call shares the one array: calls whose work overlaps on the GPU
//    (different streams, or different host threads) race on it and give
//    wrong results; serialise them;
//  - each call clears the array on its own stream before the kernel runs.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "lh_device.cuh"
#include "lh_internal.cuh"

namespace lh {
namespace {

constexpr uint32_t kNoAllocMaxTiles = 4096;
constexpr uint32_t kNoAllocWords = kNoAllocMaxTiles + 32;  // look-back words + the tile claim counter

// The scratch of every call.  Host code must not use `g_cull_scratch`
// directly: on the host it names a stand-in, not the device memory.
static __device__ __align__(256) unsigned long long g_cull_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
std::atomic<unsigned long long*> g_scratch_ptr[kMaxDevices];

__device__ __forceinline__ void na_st(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long na_ld(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Same cull and ordered append as the frame's instance cull
// (cull_instances.comp:7-27 with prefix_sum.glsl:17-30): one instance per
// thread, warp scans, decoupled look-back with bounded waits.
__global__ void __launch_bounds__(kInstTile) k_cull_instances_noalloc(const Instance* instances, uint32_t n,
                                                                    const Uniforms u, uint8_t* sector,
                                                                    uint32_t capacity, uint32_t* flags_out,
                                                                    unsigned long long* scratch) {
    __shared__ unsigned long long s_warp[kInstTile / 32];
    __shared__ unsigned long long s_excl;
    __shared__ uint32_t s_tile;
    unsigned long long* status = scratch;                         // one word per tile
    unsigned int* claim = reinterpret_cast<unsigned int*>(scratch + kNoAllocMaxTiles);
    if (threadIdx.x == 0) s_tile = atomicAdd(claim, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t i = tile * kInstTile + threadIdx.x;
    bool keep = false;
    uint32_t nm = 0;
    if (i < n) {
        const Instance* inst = instances + i;
        lh_mat4 transform;
        const float4* src = reinterpret_cast<const float4*>(inst);
        float4* dst = reinterpret_cast<float4*>(&transform);
        for (int k = 0; k < 4; k++) dst[k] = __ldg(src + k);
        const MeshInfo* mi = mesh_info_of(inst);
        const unsigned long long* w = reinterpret_cast<const unsigned long long*>(mi);
        unsigned long long w6 = __ldg(w + 6), w7 = __ldg(w + 7);
        lh_vec4 bs;
        bs.x = __uint_as_float((uint32_t)(w6 >> 32));
        bs.y = __uint_as_float((uint32_t)w7);
        bs.z = __uint_as_float((uint32_t)(w7 >> 32));
        bs.w = __uint_as_float(__ldg(reinterpret_cast<const uint32_t*>(mi) + 16));
        nm = (uint32_t)(w6 & 0xFFFFu);
        keep = !cull_bounding_sphere(u, transform, bs);
    }
    const unsigned long long pay = keep ? ((1ull << 40) | nm) : 0ull;
    unsigned long long incl = pay;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (uint32_t k = 0; k < kInstTile / 32; k++) {
            unsigned long long t = s_warp[k];
            s_warp[k] = run;
            run += t;
        }
        unsigned long long excl = 0;
        if (tile == 0) {
            na_st(&status[0], kStatIncl | run);
        } else {
            na_st(&status[tile], kStatAgg | run);
            int64_t t = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (t >= 0) {
                unsigned long long s = na_ld(&status[t]);
                unsigned long long fl = s >> 62;
                if (fl == 0) {
                    if (++spins >= kSpinLimit) {
                        // recorded by the block that timed out, whenever it does
                        if (flags_out) atomicOr(flags_out, LH_FLAG_TIMEOUT);
                        break;
                    }
                    if (spins > 32) __nanosleep(spins > 1024 ? 256 : 32);
                    continue;
                }
                excl += s & kPayloadMask;
                if (fl == 2) break;
                --t;
            }
            na_st(&status[tile], kStatIncl | (excl + run));
        }
        s_excl = excl;
        if (tile == gridDim.x - 1) {
            unsigned long long total = excl + run;
            unsigned long long count = total >> 40;
            *reinterpret_cast<unsigned long long*>(sector) = (count << 32) | (uint32_t)(total & ((1ull << 40) - 1));
            if (count > capacity) {
                if (flags_out) atomicOr(flags_out, LH_FLAG_INSTANCE_OVERFLOW);
            }
        }
    }
    __syncthreads();
    if (keep) {
        unsigned long long before = s_excl + s_warp[warp] + incl - pay;
        uint32_t pos = (uint32_t)(before >> 40);
        if (pos < capacity) {
            PrefixSumValue v;
            v.index = i;
            v.sum = (uint32_t)(before & ((1ull << 40) - 1)) + nm;
            reinterpret_cast<PrefixSumValue*>(sector + 8)[pos] = v;
        }
    }
}

// Device address of the scratch array on the current device.  Outside
// stream capture it is looked up on every call (cheap, host side only), so a
// device reset or another current context is picked up; during capture the
// address kept by the last call outside capture on this device is used.
lh_status scratch_for_current_device(cudaStream_t s, unsigned long long** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LH_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return LH_ERR_UNSUPPORTED;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return LH_ERR_CUDA;
    if (cs != cudaStreamCaptureStatusNone) {
        unsigned long long* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
        if (!p) return LH_ERR_UNSUPPORTED;  // no call outside capture on this device yet
        *out = p;
        return LH_OK;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_cull_scratch) != cudaSuccess || !addr) return LH_ERR_CUDA;
    unsigned long long* p = reinterpret_cast<unsigned long long*>(addr);
    g_scratch_ptr[dev].store(p, std::memory_order_release);
    *out = p;
    return LH_OK;
}

}  // namespace
}  // namespace lh

extern "C" lh_status lh_cull_instances_noalloc(const Instance* d_instances, uint32_t n_instances,
                                               const Uniforms* host_uniforms, uint8_t* d_sector, uint32_t capacity,
                                               uint32_t* d_flags, void* stream) {
    using namespace lh;
    if (!host_uniforms || !d_sector || (n_instances && !d_instances)) return LH_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)d_instances & 15) || ((uintptr_t)d_sector & 7)) return LH_ERR_INVALID_ARGUMENT;
    const uint32_t tiles = (n_instances + kInstTile - 1) / kInstTile;
    if (tiles > kNoAllocMaxTiles) return LH_ERR_CAPACITY;  // more than 1,048,576 instances
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long* scratch = nullptr;
    lh_status st = scratch_for_current_device(s, &scratch);
    if (st != LH_OK) return st;
    // the previous call's look-back words and claim counter must not leak in
    if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * kNoAllocWords, s) != cudaSuccess) return LH_ERR_CUDA;
    if (tiles == 0) {
        if (cudaMemsetAsync(d_sector, 0, 8, s) != cudaSuccess) return LH_ERR_CUDA;
        return LH_OK;
    }
    k_cull_instances_noalloc<<<tiles, kInstTile, 0, s>>>(d_instances, n_instances, *host_uniforms, d_sector, capacity,
                                                        d_flags, scratch);
    return cudaGetLastError() == cudaSuccess ? LH_OK : LH_ERR_CUDA;
}
