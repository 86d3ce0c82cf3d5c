// One persistent launch for the cull and raster of every view of a frame:
// the main view, the probe views and the 4 shadow cascades.
//
// The stages are the same device phases the per-stage kernels run
// (cull_phases.cuh, raster_phases.cuh, frame_phases.cuh); here one
// cooperative grid (every block resident) runs them back to back with grid
// barriers in between, so the frame's cull + raster costs one launch instead
// of ~15, and small views (probes) share the machine with the large ones in
// every phase.  The order of phases is the reference's pass order
// (src/rendering.cpp:79-438): clear, instance cull, meshlet cull, raster of
// the visibility views; depth reduction; cascade fit; instance cull, meshlet
// cull, raster of the cascades.
#include "cull_phases.cuh"
#include "frame_phases.cuh"
#include "raster_phases.cuh"
#include "waits.cuh"

namespace lh {
namespace {

// Grid barrier on a counter that only grows within the launch: barrier k
// completes when the counter reaches k * gridDim.x.  All blocks are
// resident (cooperative launch), and the wait is bounded: on expiry (or once
// another block's wait has expired) LH_FLAG_TIMEOUT is recorded and the
// barrier returns false; the kernel then stops instead of running its later
// phases on data that no barrier ordered.
__device__ bool grid_barrier(const FrameDev& f, uint32_t& epoch) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch++;
        const uint32_t target = epoch * gridDim.x;
        __threadfence();
        atomicAdd(&f.status[kStBarrier], 1u);
        const bool ok = counter_wait(&f.status[kStBarrier], target, &f.status[kStFlags], kSpinLimit);
        if (!ok) atomicOr(&f.status[kStFlags], LH_FLAG_TIMEOUT);
        __threadfence();
        s_ok = ok ? 1u : 0u;
    }
    __syncthreads();
    return s_ok != 0;
}

// Resets the raster words between the visibility and the shadow passes.
__device__ void reset_raster_words(const FrameDev& f) {
    for (uint32_t w = kStClipCount + threadIdx.x; w <= kStRasterClaimAlpha; w += blockDim.x)
        if (w != kStBarrier && w != kStReduceDone) f.status[w] = 0u;
}

constexpr int kPersistentThreads = 256;

__global__ void __launch_bounds__(kPersistentThreads, 3) k_frame_persistent(FrameDev f, uint32_t n_persp,
                                                                           RasterTune tune) {
    __shared__ RasterSmemAlpha s_raster;  // reused by every raster phase
    uint32_t epoch = 0;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, gstride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t n_views = n_persp + 4;
    // clear every target; block 0 resets the per-view counters and the depth range
    for (uint32_t v = 0; v < n_views; v++) phase_clear_view(f, v, gtid, gstride, blockIdx.x == 0 && v == 0);
    if (!grid_barrier(f, epoch)) return;
    const uint32_t inst_tiles = (f.n_instances + kInstTile - 1) / kInstTile;
    // visibility views: instance cull + prefix sum
    for (uint32_t vb = blockIdx.x; vb < inst_tiles * n_persp; vb += gridDim.x)
        phase_cull_instances_tile(f, vb / inst_tiles, inst_tiles);
    if (!grid_barrier(f, epoch)) return;
    phase_cull_meshlets(f, 0, n_persp, &f.status[kStMlClaim]);
    if (!grid_barrier(f, epoch)) return;
    if (f.occlusion_px) {
        // occluders and their chunks, hierarchical depth, the depth test of
        // the other meshlets, then the survivors
        phase_raster<0, false>(f, 0, n_persp, tune, &f.status[kStRasterClaim], s_raster, nullptr, kListOccluders);
        if (!grid_barrier(f, epoch)) return;
        phase_raster_big<0>(f);
        if (!grid_barrier(f, epoch)) return;
        phase_hiz(f, 0, n_persp);
        if (!grid_barrier(f, epoch)) return;
        phase_occlusion_filter(f, 0, n_persp, gtid, gstride);
        if (!grid_barrier(f, epoch)) return;
        phase_raster<0, false>(f, 0, n_persp, tune, &f.status[kStRasterClaim], s_raster, nullptr, kListSurvivors);
        phase_raster<0, true>(f, 0, n_persp, tune, &f.status[kStRasterClaimAlpha], s_raster, s_raster.av,
                              kListSurvivors);
    } else {
        phase_raster<0, false>(f, 0, n_persp, tune, &f.status[kStRasterClaim], s_raster, nullptr);
        phase_raster<0, true>(f, 0, n_persp, tune, &f.status[kStRasterClaimAlpha], s_raster, s_raster.av);
    }
    if (!grid_barrier(f, epoch)) return;
    phase_raster_big<0>(f);
    if (!grid_barrier(f, epoch)) return;
    // depth range of the main view, then the cascade fit
    phase_depth_reduce(f, gtid, gstride);
    if (!grid_barrier(f, epoch)) return;
    if (blockIdx.x == 0) {
        phase_fit(f);
        reset_raster_words(f);
    }
    if (!grid_barrier(f, epoch)) return;
    // cascades
    for (uint32_t vb = blockIdx.x; vb < inst_tiles * 4; vb += gridDim.x)
        phase_cull_instances_tile(f, n_persp + vb / inst_tiles, inst_tiles);
    if (!grid_barrier(f, epoch)) return;
    phase_cull_meshlets(f, n_persp, 4, &f.status[kStMlClaim]);
    if (!grid_barrier(f, epoch)) return;
    phase_raster<1, false>(f, n_persp, 4, tune, &f.status[kStRasterClaim], s_raster, nullptr);
    phase_raster<1, true>(f, n_persp, 4, tune, &f.status[kStRasterClaimAlpha], s_raster, s_raster.av);
    if (!grid_barrier(f, epoch)) return;
    phase_raster_big<1>(f);
}

int g_persistent_blocks_per_sm = -1;

}  // namespace

// Blocks per SM at which the persistent kernel is resident (0 if it cannot be).
int persistent_blocks_per_sm() {
    if (g_persistent_blocks_per_sm < 0) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_frame_persistent, kPersistentThreads, 0) != cudaSuccess)
            n = 0;
        g_persistent_blocks_per_sm = n;
    }
    return g_persistent_blocks_per_sm;
}

cudaError_t launch_frame_persistent(const FrameDev& f, uint32_t n_persp, uint32_t small_px, uint32_t medium_px,
                                    uint32_t raster_batch,
                                    float blocks_per_sm, cudaStream_t s, int sms) {
    const int resident = persistent_blocks_per_sm();
    if (resident <= 0) return cudaErrorCooperativeLaunchTooLarge;
    (void)blocks_per_sm;
    const int per_sm = resident;  // every resident slot: the raster phases need the occupancy
    RasterTune tune{small_px, medium_px, raster_batch};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sms * per_sm));
    cfg.blockDim = dim3(kPersistentThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_frame_persistent, f, n_persp, tune);
}

}  // namespace lh
