// Kernels of the instance cull + single-pass prefix sum and of the meshlet
// cull; the work itself is in cull_phases.cuh (shared with the persistent
// multi-view kernel).
#include "cull_phases.cuh"
#include "frame_phases.cuh"

namespace lh {
namespace {

// grid = (tiles per view + clear blocks, n_views).  Blocks past the view's
// tiles clear its target (visibility 0 or shadow depth 1.0) while the tiles
// cull: the cull occupies few SMs, and nothing reads the target before the
// raster launched after it.  Also zeroes the claim word of the meshlet cull
// that follows in the stream (nothing here reads it).
__global__ void __launch_bounds__(kInstTile) k_cull_instances(FrameDev f, uint32_t view_begin, uint32_t tiles) {
    pdl_enter();
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) f.status[kStMlClaim] = 0u;
    if (blockIdx.x >= tiles) {
        const uint32_t clear_blocks = gridDim.x - tiles;
        phase_clear_view(f, view_begin + blockIdx.y, (uint64_t)(blockIdx.x - tiles) * blockDim.x + threadIdx.x,
                         (uint64_t)clear_blocks * blockDim.x, false);
        return;
    }
    phase_cull_instances_tile(f, view_begin + blockIdx.y, tiles);
}

// persistent over (view, tile) claims of views [view_begin, view_begin + n_views).
// Also zeroes the raster words of the raster launches that follow (clip
// count, claims, reduce counter, big-triangle counter; nothing here reads
// them).
// Registers bounded for LH_ML_MIN_BLOCKS resident blocks per SM (build knob):
// the launch's blocks (lh_tuning.cull_blocks_per_sm per SM, 3 by default)
// then all run at once, one 512-candidate tile after another.
#ifndef LH_ML_MIN_BLOCKS
#define LH_ML_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(kMlThreads, LH_ML_MIN_BLOCKS)
    k_cull_meshlets(FrameDev f, uint32_t view_begin, uint32_t n_views) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x < kStWords) {
        const uint32_t w = threadIdx.x;
        if (w >= kStClipCount && w <= kStRasterClaimAlpha && w != kStMlClaim && w != kStBarrier) f.status[w] = 0u;
    }
    phase_cull_meshlets(f, view_begin, n_views, &f.status[kStMlClaim]);
}

// out[0]: the scene's meshlets; out[1] (low word): the OR of its meshes' flags.
__global__ void k_sum_meshlets(const Instance* inst, uint32_t n, unsigned long long* out) {
    unsigned long long acc = 0;
    uint32_t flags = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const MeshInfoCull mi = load_mesh_info(mesh_info_of(inst + i));
        acc += mi.num_meshlets;
        flags |= mi.flags;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, acc);
        atomicOr(reinterpret_cast<unsigned int*>(out + 1), flags);
    }
}

}  // namespace

cudaError_t launch_cull_instances(const FrameDev& f, uint32_t view_begin, uint32_t n_views, cudaStream_t s,
                                  uint32_t clear_blocks) {
    if (n_views == 0) return cudaSuccess;
    const uint32_t tiles = (f.n_instances + kInstTile - 1) / kInstTile;
    if (tiles + clear_blocks == 0) return cudaSuccess;
    dim3 grid(tiles + clear_blocks, n_views);
    return launch_pdl(k_cull_instances, grid, dim3(kInstTile), s, f, view_begin, tiles);
}

cudaError_t launch_cull_meshlets(const FrameDev& f, uint32_t view_begin, uint32_t n_views, uint32_t blocks,
                                 cudaStream_t s) {
    if (n_views == 0) return cudaSuccess;
    // the claim word was zeroed by the frame start or the instance cull
    return launch_pdl(k_cull_meshlets, dim3(blocks), dim3(kMlThreads), s, f, view_begin, n_views);
}

cudaError_t launch_sum_meshlets(const Instance* instances, uint32_t n, unsigned long long* out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess || n == 0) return e;
    k_sum_meshlets<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, s>>>(instances, n, out);
    return cudaGetLastError();
}

}  // namespace lh
