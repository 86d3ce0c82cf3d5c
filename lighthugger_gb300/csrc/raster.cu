// Kernels of the compute rasteriser; the work itself is in raster_phases.cuh
// (shared with the persistent multi-view kernel).
#include "raster_phases.cuh"

#ifndef LH_RASTER_MIN_BLOCKS
#define LH_RASTER_MIN_BLOCKS 3  // resident blocks of k_raster per SM (registers: 65536 / 256 / this)
#endif
#ifndef LH_RASTER_MULTIVIEW_MIN_BLOCKS
#define LH_RASTER_MULTIVIEW_MIN_BLOCKS 4  // the same when one launch rasterises several visibility views
#endif
#ifndef LH_RASTER_BIG_MIN_BLOCKS
#define LH_RASTER_BIG_MIN_BLOCKS 4  // the same for the chunk kernel k_raster_big
#endif

namespace lh {
namespace {

// MINB resident blocks per SM.  One large view (the main visibility view,
// the cascades) runs best at 3 (80 registers, no spills); a launch over many
// small views (main + probes: mostly meshlets whose vertices span no pixel
// centre, bound by the latency of their loads) at 4 (64 registers): 3.66 ->
// 3.53 ms for main + 32 probes + 4 cascades, while 4 costs the lone main
// view 0.328 -> 0.343 ms.
template <int KIND, int MINB>
__global__ void __launch_bounds__(kRasterWarps * 32, MINB) k_raster(FrameDev f, uint32_t view_begin, uint32_t n_views,
                                                                   RasterTune tune, uint32_t list) {
    __shared__ RasterSmem sm;
    pdl_enter();
    phase_raster<KIND, false>(f, view_begin, n_views, tune, &f.status[kStRasterClaim], sm, nullptr, list);
}

// The alpha-clip draw class (double sided, alpha tested).
template <int KIND>
__global__ void __launch_bounds__(kRasterWarps * 32, 3) k_raster_alpha(FrameDev f, uint32_t view_begin,
                                                                       uint32_t n_views, RasterTune tune, uint32_t list) {
    __shared__ RasterSmemAlpha sm;
    pdl_enter();
    phase_raster<KIND, true>(f, view_begin, n_views, tune, &f.status[kStRasterClaimAlpha], sm, sm.av, list);
}

template <int KIND>
__global__ void __launch_bounds__(256, LH_RASTER_BIG_MIN_BLOCKS) k_raster_big(FrameDev f) {
    pdl_enter();
    phase_raster_big<KIND>(f);
}

// Hierarchical depth of the visibility views after the occluder pass.
__global__ void __launch_bounds__(256) k_hiz(FrameDev f, uint32_t view_begin, uint32_t n_views) {
    pdl_enter();
    phase_hiz(f, view_begin, n_views);
}

// Depth test of the other visible meshlets' spheres; survivor lists.
__global__ void __launch_bounds__(256) k_occlusion_filter(FrameDev f, uint32_t view_begin, uint32_t n_views) {
    pdl_enter();
    phase_occlusion_filter(f, view_begin, n_views, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                           (uint64_t)gridDim.x * blockDim.x);
}

}  // namespace

cudaError_t launch_raster_kind(const FrameDev& f, uint32_t view_begin, uint32_t n_views, int kind, uint32_t small_px,
                               uint32_t medium_px, uint32_t raster_batch, cudaStream_t s, int sms) {
    if (n_views == 0) return cudaSuccess;
    if (n_views > kMaxViews) return cudaErrorInvalidValue;
    RasterTune tune{small_px, medium_px, raster_batch};
    // the raster words (clip count, claims, reduce counter, packed
    // big-triangle word) were zeroed by the meshlet cull launched before
    const dim3 rb(kRasterWarps * 32);
    cudaError_t e;
    if (kind == kViewVisibility) {
        auto opaque = [&](uint32_t list) {
            if (n_views > 1)
                return launch_pdl(k_raster<0, LH_RASTER_MULTIVIEW_MIN_BLOCKS>,
                                  dim3(sms * LH_RASTER_MULTIVIEW_MIN_BLOCKS), rb, s, f, view_begin, n_views, tune, list);
            return launch_pdl(k_raster<0, LH_RASTER_MIN_BLOCKS>, dim3(sms * LH_RASTER_MIN_BLOCKS), rb, s, f, view_begin,
                              n_views, tune, list);
        };
        const dim3 big_grid(sms * LH_RASTER_BIG_MIN_BLOCKS);
        if (f.occlusion_px) {
            // occluders (and their chunks), hierarchical depth, the depth
            // test of every other meshlet, then the survivors
            e = opaque(kListOccluders);
            if (e == cudaSuccess) e = launch_pdl(k_raster_big<0>, big_grid, dim3(256), s, f);
            if (e == cudaSuccess) e = launch_pdl(k_hiz, dim3(sms * 4), dim3(256), s, f, view_begin, n_views);
            if (e == cudaSuccess)
                e = launch_pdl(k_occlusion_filter, dim3(sms * 8), dim3(256), s, f, view_begin, n_views);
            if (e == cudaSuccess) e = opaque(kListSurvivors);
            if (e == cudaSuccess && f.scene_alpha)
                e = launch_pdl(k_raster_alpha<0>, dim3(sms * 3), rb, s, f, view_begin, n_views, tune,
                               (uint32_t)kListSurvivors);
        } else {
            e = opaque(kListAll);
            if (e == cudaSuccess && f.scene_alpha)
                e = launch_pdl(k_raster_alpha<0>, dim3(sms * 3), rb, s, f, view_begin, n_views, tune,
                               (uint32_t)kListAll);
        }
        if (e == cudaSuccess) e = launch_pdl(k_raster_big<0>, big_grid, dim3(256), s, f);
    } else {
        e = launch_pdl(k_raster<1, LH_RASTER_MIN_BLOCKS>, dim3(sms * LH_RASTER_MIN_BLOCKS), rb, s, f, view_begin, n_views,
                       tune, (uint32_t)kListAll);
        if (e == cudaSuccess && f.scene_alpha)
            e = launch_pdl(k_raster_alpha<1>, dim3(sms * 3), rb, s, f, view_begin, n_views, tune, (uint32_t)kListAll);
        if (e == cudaSuccess) e = launch_pdl(k_raster_big<1>, dim3(sms * LH_RASTER_BIG_MIN_BLOCKS), dim3(256), s, f);
    }
    return e;
}

}  // namespace lh
