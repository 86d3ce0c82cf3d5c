// C ABI of the visibility pipeline: context, buffers and the stream-ordered
// frame that replaces src/rendering.cpp:28-474 (render()).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lh/lh.h"
#include "lh_internal.cuh"

using namespace lh;

namespace {

constexpr uint32_t kVersion = 1;

// The resolve adjoint captured with a graphed frame (all zero: none).
struct GraphBackward {
    uint64_t grad;
    lh_grad_targets targets;
};

struct Alloc {
    void* p = nullptr;
    size_t bytes = 0;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr size_t kConstBytes = 64;  // frame constants ahead of the Uniforms (device and staging)

}  // namespace

struct lh_ctx {
    lh_config cfg{};
    int device = 0;
    int sms = 0;
    std::string err;
    std::vector<Alloc> allocs;
    // fixed buffers
    Uniforms* d_uniforms = nullptr;  // [0] main, [1..max_probes] probes
    float* d_consts = nullptr;       // frame constants
    float* d_srgb = nullptr;
    MiscStorage* d_misc = nullptr;
    uint32_t* d_status = nullptr;
    uint8_t* d_sectors = nullptr;
    MeshletReference* d_refs = nullptr;
    RasterDraw* d_rdraws = nullptr;  // the raster's per-slot draw records
    uint32_t* d_lists = nullptr;     // occlusion lists of the visibility views (3 * max_draws words each)
    uint32_t* d_hiz = nullptr;       // hierarchical depth of the visibility views (pool)
    size_t hiz_words = 0;
    uint8_t* d_draws = nullptr;
    uint64_t* d_vis = nullptr;
    float* d_shadow = nullptr;
    void* d_hdr = nullptr;
    uint64_t* d_probe_vis = nullptr;
    BigTri* d_big = nullptr;
    uint32_t* d_big_base = nullptr;
    ViewDev* d_views = nullptr;
    lh_texture* d_textures = nullptr;
    uint32_t n_textures = 0;
    // linear float4 copies of the textures (one buffer) and a table of
    // device pointers into it, made by lh_set_scene
    float4* d_tex_linear = nullptr;
    const float4** d_tex_linear_ptrs = nullptr;
    std::vector<size_t> tex_offset;    // first texel of each texture in d_tex_linear (n_textures + 1)
    std::vector<uint32_t> tex_size;    // width, height of each texture
    // per-frame zeroed scratch (look-back words and tile claims)
    uint8_t* d_reset = nullptr;
    size_t reset_bytes = 0;
    size_t sector_bytes = 0, draw_bytes = 0;
    uint32_t max_views = 0;
    // scene
    const Instance* instances = nullptr;
    uint32_t n_instances = 0;
    uint64_t scene_meshlets = 0;
    // host staging for per-frame constants (pinned, double buffered)
    uint8_t* h_staging[2] = {nullptr, nullptr};
    cudaEvent_t staging_done[2] = {nullptr, nullptr};
    size_t staging_bytes = 0;
    uint32_t frame_index = 0;
    uint32_t n_views_last = 5;
    uint32_t n_probes_last = 0;
    cudaStream_t last_stream = nullptr;
    std::vector<ViewDev> h_views;
    lh_tuning tuning{};
    // stage timing
    bool profiling = false;
    cudaEvent_t stage_ev[LH_N_STAGES + 1] = {};
    // graph (plain frames keep the template graph and its frame-start node,
    // whose kernel parameters carry each replay's uniforms)
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph_template = nullptr;
    bool scene_alpha = true;  // some mesh is alpha clip (lh_set_scene)
    cudaGraphNode_t graph_clear_node = nullptr;
    uint32_t graph_probes = 0;
    uint32_t graph_instances = 0;
    lh_tuning graph_tuning{};
    cudaStream_t capture_stream = nullptr;
    bool capturing = false;
    GraphBackward graph_backward{};
    bool graph_until_resolve = false;
    float4* d_lut_standin = nullptr;  // identity 48^3 LUT for lh_display_transform
    // 2D tensor map of d_vis for the TMA-staged resolve (false: rows are not
    // 16-byte aligned or the driver lacks the encoder)
    CUtensorMap vis_map;  // the type carries its own (TMA) alignment
    bool vis_map_ok = false;
    // pipelined HDR readback (lh_frame_readback): copies on their own
    // stream; a frame's resolve waits for the previous copy of d_hdr
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t resolved = nullptr;
    cudaEvent_t readback_done[2] = {nullptr, nullptr};
    uint32_t readbacks = 0;
};

namespace {

// Tensor map of the main visibility buffer: u64 elements, W x H, boxes of
// 128 x 1 (one warp's row of a resolve strip).  cuTensorMapEncodeTiled is reached through
// the runtime's driver entry point, so nothing links against libcuda.
bool encode_vis_map(lh_ctx* c) {
    const uint64_t W = c->cfg.width, H = c->cfg.height;
    if ((W * 8) % 16 != 0) return false;
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return false;
    const cuuint64_t dims[2] = {W, H};
    const cuuint64_t strides[1] = {W * 8};
    const cuuint32_t box[2] = {128, 1};
    const cuuint32_t elem[2] = {1, 1};
    return reinterpret_cast<Encode>(fn)(&c->vis_map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, c->d_vis, dims, strides, box,
                                        elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

lh_status fail(lh_ctx* c, lh_status st, const std::string& msg) {
    if (c) c->err = msg;
    return st;
}

lh_status cuda_fail(lh_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? LH_ERR_OUT_OF_MEMORY : LH_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
cudaError_t dalloc(lh_ctx* c, T** out, size_t bytes) {
    void* p = nullptr;
    size_t b = align_up(std::max<size_t>(bytes, 16), 256);
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) return e;
    c->allocs.push_back({p, b});
    *out = reinterpret_cast<T*>(p);
    return cudaSuccess;
}

void drop_graph(lh_ctx* c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
    if (c->graph_template) cudaGraphDestroy(c->graph_template);
    c->graph_template = nullptr;
    c->graph_clear_node = nullptr;
}

void free_all(lh_ctx* c) {
    for (auto& ev : c->stage_ev)
        if (ev) { cudaEventDestroy(ev); ev = nullptr; }
    drop_graph(c);
    if (c->capture_stream) cudaStreamDestroy(c->capture_stream);
    c->capture_stream = nullptr;
    for (auto& a : c->allocs) cudaFree(a.p);
    c->allocs.clear();
    for (int i = 0; i < 2; i++) {
        if (c->h_staging[i]) cudaFreeHost(c->h_staging[i]);
        if (c->staging_done[i]) cudaEventDestroy(c->staging_done[i]);
        if (c->readback_done[i]) cudaEventDestroy(c->readback_done[i]);
        c->h_staging[i] = nullptr;
        c->staging_done[i] = nullptr;
        c->readback_done[i] = nullptr;
    }
    if (c->resolved) cudaEventDestroy(c->resolved);
    c->resolved = nullptr;
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    c->copy_stream = nullptr;
}

size_t hdr_pixel_bytes(const lh_config& cfg) { return (cfg.flags & LH_CONFIG_HDR_RGBA16F) ? 8 : 16; }

// Work that writes d_hdr waits for the last pipelined readback of it.
cudaError_t wait_readback(const lh_ctx* c, cudaStream_t s) {
    if (!c->readbacks) return cudaSuccess;
    return cudaStreamWaitEvent(s, c->readback_done[(c->readbacks - 1) & 1u], 0);
}

// View order: 0 main, 1..n_probes probes, then cascades 0..3.
void build_views(lh_ctx* c, uint32_t n_probes, const Uniforms* probe_uniforms) {
    const lh_config& cfg = c->cfg;
    c->h_views.clear();
    size_t probe_off = 0;
    uint32_t n_views = 5 + n_probes;
    uint32_t n_inst_tiles = (c->n_instances + kInstTile - 1) / kInstTile + 1;
    uint32_t ml_tiles = (uint32_t)((c->scene_meshlets + kMlTile - 1) / kMlTile) + 1;
    size_t per_view = align_up(4 * kClaimWords + 8 * (size_t)n_inst_tiles + 8 * (size_t)ml_tiles, 256);
    size_t hiz_used = 0;
    for (uint32_t v = 0; v < n_views; v++) {
        ViewDev vw{};
        bool cascade = v >= 1 + n_probes;
        vw.kind = cascade ? kViewShadow : kViewVisibility;
        vw.cascade = cascade ? v - 1 - n_probes : 0;
        if (v == 0) {
            vw.width = cfg.width;
            vw.height = cfg.height;
            vw.target = c->d_vis;
            vw.uniforms = c->d_uniforms;
        } else if (!cascade) {
            const Uniforms& pu = probe_uniforms[v - 1];
            vw.width = pu.window_size.x;
            vw.height = pu.window_size.y;
            vw.target = c->d_probe_vis + probe_off;
            probe_off += align_up((size_t)vw.width * vw.height, 32);
            vw.uniforms = c->d_uniforms + v;
        } else {
            vw.width = vw.height = cfg.shadow_size;
            vw.target = c->d_shadow + (size_t)vw.cascade * cfg.shadow_size * cfg.shadow_size;
            vw.uniforms = c->d_uniforms;
        }
        vw.sector = c->d_sectors + v * c->sector_bytes;
        vw.refs = c->d_refs + (size_t)v * 2 * cfg.max_draws;
        vw.rdraws = c->d_rdraws + (size_t)v * 2 * cfg.max_draws;
        vw.draws = c->d_draws + v * c->draw_bytes;
        vw.section_base = v * 2 * cfg.max_draws;
        uint8_t* r = c->d_reset + kStWords * 4 + v * per_view;
        vw.claim = reinterpret_cast<uint32_t*>(r);
        vw.inst_status = reinterpret_cast<uint64_t*>(r + 4 * kClaimWords);
        vw.ml_status = reinterpret_cast<uint64_t*>(r + 4 * kClaimWords + 8 * (size_t)n_inst_tiles);
        vw.ml_tile_cap = ml_tiles;
        if (!cascade) {
            // occlusion lists, and the view's hierarchical depth from the
            // pool while it lasts (a view without one culls nothing)
            vw.lists = c->d_lists + (size_t)v * 3 * cfg.max_draws;
            vw.hiz_rx = (vw.width + kHizRegion - 1) / kHizRegion;
            vw.hiz_ry = (vw.height + kHizRegion - 1) / kHizRegion;
            const size_t words = (size_t)vw.hiz_rx * vw.hiz_ry * 65;
            if (hiz_used + words <= c->hiz_words) {
                vw.hiz = c->d_hiz + hiz_used;
                hiz_used += align_up(words, 64);
            }
        }
        c->h_views.push_back(vw);
    }
}

size_t reset_bytes_for(const lh_ctx* c) {
    uint32_t n_inst_tiles = (c->n_instances + kInstTile - 1) / kInstTile + 1;
    uint32_t ml_tiles = (uint32_t)((c->scene_meshlets + kMlTile - 1) / kMlTile) + 1;
    size_t per_view = align_up(4 * kClaimWords + 8 * (size_t)n_inst_tiles + 8 * (size_t)ml_tiles, 256);
    return align_up(kStWords * 4, 256) + per_view * c->max_views;
}

FrameDev frame_dev(const lh_ctx* c, uint32_t n_views, uint32_t n_instances) {
    FrameDev f{};
    f.instances = c->instances;
    f.n_instances = n_instances;
    f.max_instances = c->cfg.max_instances;
    f.max_draws = c->cfg.max_draws;
    f.n_views = n_views;
    f.misc = c->d_misc;
    f.status = reinterpret_cast<uint32_t*>(c->d_reset);
    f.views = c->d_views;
    f.big = c->d_big;
    f.big_base = c->d_big_base;
    f.big_cap = c->cfg.max_big_triangles;
    f.textures = c->d_textures;
    f.n_textures = c->n_textures;
    f.tex_linear = c->d_tex_linear_ptrs;
    f.shadow_maps = c->d_shadow;
    f.shadow_size = c->cfg.shadow_size;
    f.hdr = c->d_hdr;
    f.hdr_half = (c->cfg.flags & LH_CONFIG_HDR_RGBA16F) ? 1u : 0u;
    f.visibility = c->d_vis;
    f.uniforms = c->d_uniforms;
    f.frame_consts = c->d_consts;
    f.srgb_lut = c->d_srgb;
    f.occlusion_px = c->tuning.occlusion_px;
    f.scene_alpha = c->scene_alpha ? 1u : 0u;
    for (int k = 0; k < 2; k++) {
        f.chunk_shift[k][0] = (uint32_t)__builtin_ctz(c->tuning.chunk_rows[k]);
        f.chunk_shift[k][1] = (uint32_t)__builtin_ctz(c->tuning.chunk_cols[k]);
    }
    f.backward_rows = c->tuning.backward_rows;
    return f;
}

lh_status check_ctx(lh_ctx* c) {
    if (!c) return LH_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    return LH_OK;
}

// Stage per-frame constants (uniforms + host-evaluated pow terms) in pinned
// memory and copy them to the device on `s`.
// The per-frame Uniforms as the kernels read them (address fields are the
// context's own buffers) and the frame constants.
void fill_frame_constants(const lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes, Uniforms* hu,
                          float* consts) {
    hu[0] = *u;
    for (uint32_t p = 0; p < n_probes; p++) hu[1 + p] = probes[p];
    for (uint32_t v = 0; v <= n_probes; v++) {
        hu[v].meshlet_references = (uint64_t)(uintptr_t)c->h_views[v].refs;
        hu[v].instances = (uint64_t)(uintptr_t)c->instances;
        hu[v].draw_calls = (uint64_t)(uintptr_t)c->h_views[v].draws;
        hu[v].misc_storage = (uint64_t)(uintptr_t)c->d_misc;
        hu[v].num_meshlets_prefix_sum = (uint64_t)(uintptr_t)c->h_views[v].sector;
        hu[v].dispatches = 0;
    }
    // generate_shadow_matrices.glsl:39-48: pow(0.5|0.75, cascade_split_pow),
    // uniform-only terms, evaluated here in double and rounded to float.
    consts[0] = (float)std::pow(0.5, (double)u->cascade_split_pow);
    consts[1] = (float)std::pow(0.75, (double)u->cascade_split_pow);
}

// A plain frame's start parameters: the main view's uniforms and frame
// constants, and the per-frame scratch the frame-start kernel zeroes.
FrameStart make_frame_start(lh_ctx* c, const Uniforms* u) {
    FrameStart start;
    std::memset(&start, 0, sizeof(start));
    fill_frame_constants(c, u, nullptr, 0, &start.u, start.consts);
    start.d_uniforms = c->d_uniforms;
    start.d_consts = c->d_consts;
    start.reset = reinterpret_cast<uint4*>(c->d_reset);
    start.reset_words = c->reset_bytes / sizeof(uint4);
    return start;
}

lh_status upload_frame_constants(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes,
                                 cudaStream_t s) {
    uint32_t slot = c->frame_index++ & 1u;
    cudaError_t e = cudaEventSynchronize(c->staging_done[slot]);
    if (e != cudaSuccess) return cuda_fail(c, e, "staging event");
    // staging and device share one layout: 64 bytes of frame constants, then
    // the views' Uniforms -- one copy per frame
    uint8_t* h = c->h_staging[slot];
    fill_frame_constants(c, u, probes, n_probes, reinterpret_cast<Uniforms*>(h + kConstBytes),
                         reinterpret_cast<float*>(h));
    const size_t bytes = kConstBytes + sizeof(Uniforms) * (1 + n_probes);
    e = cudaMemcpyAsync(c->d_consts, h, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(c->staging_done[slot], s);
    if (e != cudaSuccess) return cuda_fail(c, e, "upload uniforms");
    return LH_OK;
}

// The frame's kernels, all stream ordered (capturable).  The default is the
// per-stage schedule for every frame: with the multi-view raster at four
// blocks per SM it measured 3.15 ms against 3.22 ms for the persistent
// launch on main + 32 probes + 4 cascades at 2048^2.  `batched` (a frame with
// probe views) is kept for schedules that depend on it.
uint32_t frame_schedule(const lh_ctx* c, bool batched) {
    (void)batched;
    uint32_t schedule = c->tuning.schedule;
    if (schedule == LH_SCHEDULE_DEFAULT) schedule = LH_SCHEDULE_PER_STAGE;
    if (schedule == LH_SCHEDULE_PERSISTENT && persistent_blocks_per_sm() <= 0) schedule = LH_SCHEDULE_PER_STAGE;
    return schedule;
}

// `start` (schedules with a clear launch only): the uniforms, constants and
// scratch reset travel with the clear kernel instead of copies and a memset.
// `with_resolve` false: everything up to the resolve (the caller launches it).
lh_status enqueue_frame(lh_ctx* c, uint32_t n_probes, uint32_t n_instances, bool batched, cudaStream_t s,
                        const FrameStart* start = nullptr, bool with_resolve = true) {
    const uint32_t n_persp = 1 + n_probes, n_views = n_persp + 4;
    FrameDev f = frame_dev(c, n_views, n_instances);
    const lh_tuning& t = c->tuning;
    const uint32_t schedule = frame_schedule(c, batched && n_probes > 0);
    if (start && schedule == LH_SCHEDULE_PERSISTENT) return fail(c, LH_ERR_CUDA, "frame start without a clear launch");
    const bool prof = c->profiling && !c->capturing;
    uint32_t stage = 0;
    auto mark = [&](cudaError_t e) {
        if (e == cudaSuccess && prof) e = cudaEventRecord(c->stage_ev[stage], s);
        stage++;
        return e;
    };
    auto skip_to = [&](uint32_t k, cudaError_t e) {  // stages fused into one launch share a mark
        while (e == cudaSuccess && stage < k) e = mark(e);
        return e;
    };
    cudaError_t e = mark(cudaSuccess);
    if (e == cudaSuccess && !start) e = cudaMemsetAsync(c->d_reset, 0, c->reset_bytes, s);
    const uint32_t cull_blocks = std::max(1u, (uint32_t)(c->sms * t.cull_blocks_per_sm));
    const uint32_t clear_blocks = (uint32_t)c->sms;  // per view, beside each instance-cull launch
    if (schedule == LH_SCHEDULE_PERSISTENT) {
        // stages 0..7 in one launch: the time lands in stage 0 ("clear")
        if (e == cudaSuccess)
            e = launch_frame_persistent(f, n_persp, t.small_px, t.medium_px, t.raster_batch, t.cull_blocks_per_sm, s,
                                        c->sms);
        e = mark(e);
        e = skip_to(8, e);
    } else if (schedule == LH_SCHEDULE_PER_VIEW) {
        if (e == cudaSuccess) e = mark(launch_clear_targets(f, s, c->sms, start, false));
        for (uint32_t v = 0; v < n_persp && e == cudaSuccess; v++) {
            e = launch_cull_instances(f, v, 1, s, clear_blocks);
            if (e == cudaSuccess) e = launch_cull_meshlets(f, v, 1, cull_blocks, s);
            if (e == cudaSuccess)
                e = launch_raster_kind(f, v, 1, kViewVisibility, t.small_px, t.medium_px, t.raster_batch, s, c->sms);
        }
        e = skip_to(4, e);
        if (e == cudaSuccess) e = mark(launch_depth_reduce_fit(f, s, c->sms));
        for (uint32_t k = 0; k < 4 && e == cudaSuccess; k++) {
            e = launch_cull_instances(f, n_persp + k, 1, s, clear_blocks);
            if (e == cudaSuccess) e = launch_cull_meshlets(f, n_persp + k, 1, cull_blocks, s);
            if (e == cudaSuccess)
                e = launch_raster_kind(f, n_persp + k, 1, kViewShadow, t.small_px, t.medium_px, t.raster_batch, s, c->sms);
        }
        e = skip_to(8, e);
    } else {
        if (e == cudaSuccess) e = mark(launch_clear_targets(f, s, c->sms, start, false));
        // visibility views: instance cull + prefix (and the targets' clear), meshlet cull, raster
        if (e == cudaSuccess) e = mark(launch_cull_instances(f, 0, n_persp, s, clear_blocks));
        if (e == cudaSuccess) e = mark(launch_cull_meshlets(f, 0, n_persp, cull_blocks, s));
        if (e == cudaSuccess)
            e = mark(launch_raster_kind(f, 0, n_persp, kViewVisibility, t.small_px, t.medium_px, t.raster_batch, s, c->sms));
        // depth range + cascade fit (main view only)
        if (e == cudaSuccess) e = mark(launch_depth_reduce_fit(f, s, c->sms));
        // cascades (the shadow maps are cleared beside their instance cull)
        if (e == cudaSuccess) e = mark(launch_cull_instances(f, n_persp, 4, s, clear_blocks));
        if (e == cudaSuccess) e = mark(launch_cull_meshlets(f, n_persp, 4, cull_blocks, s));
        if (e == cudaSuccess)
            e = mark(launch_raster_kind(f, n_persp, 4, kViewShadow, t.small_px, t.medium_px, t.raster_batch, s, c->sms));
    }
    // lighting resolve of the main view (after the last pipelined readback
    // of the image it overwrites; a captured graph waits as a whole instead)
    if (with_resolve) {
        if (e == cudaSuccess && !c->capturing) e = wait_readback(c, s);
        if (e == cudaSuccess)
            e = mark(launch_resolve(f, c->cfg.width, c->cfg.height, c->vis_map_ok ? &c->vis_map : nullptr, s, c->sms));
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "frame launch");
    return LH_OK;
}

lh_status prepare_views(lh_ctx* c, const Uniforms* probes, uint32_t n_probes) {
    build_views(c, n_probes, probes);
    cudaError_t e = cudaMemcpy(c->d_views, c->h_views.data(), sizeof(ViewDev) * c->h_views.size(),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "views upload");
    c->n_views_last = (uint32_t)c->h_views.size();
    c->n_probes_last = n_probes;
    return LH_OK;
}

void fill_out(const lh_ctx* c, lh_frame_out* o) {
    std::memset(o, 0, sizeof(*o));
    o->visibility = (uint64_t)(uintptr_t)c->d_vis;
    o->hdr = (uint64_t)(uintptr_t)c->d_hdr;
    o->shadow_maps = (uint64_t)(uintptr_t)c->d_shadow;
    o->misc_storage = (uint64_t)(uintptr_t)c->d_misc;
    o->prefix_sums = (uint64_t)(uintptr_t)c->d_sectors;
    o->meshlet_references = (uint64_t)(uintptr_t)c->d_refs;
    o->draw_calls = (uint64_t)(uintptr_t)c->d_draws;
    o->probe_visibility = (uint64_t)(uintptr_t)c->d_probe_vis;
    o->prefix_sector_bytes = c->sector_bytes;
    o->draw_call_section_bytes = c->draw_bytes;
    o->width = c->cfg.width;
    o->height = c->cfg.height;
    o->shadow_size = c->cfg.shadow_size;
    o->max_instances = c->cfg.max_instances;
    o->max_draws = c->cfg.max_draws;
    o->n_views = c->n_views_last;
    o->n_probes = c->n_probes_last;
}

lh_status validate_probes(lh_ctx* c, const Uniforms* probes, uint32_t n_probes) {
    if (n_probes > c->cfg.max_probes) return fail(c, LH_ERR_CAPACITY, "more probes than max_probes");
    if (n_probes && !probes) return fail(c, LH_ERR_INVALID_ARGUMENT, "probe_uniforms is NULL");
    uint64_t px = 0;
    for (uint32_t p = 0; p < n_probes; p++) {
        if (probes[p].window_size.x == 0 || probes[p].window_size.y == 0)
            return fail(c, LH_ERR_INVALID_ARGUMENT, "probe with an empty window");
        px += align_up((size_t)probes[p].window_size.x * probes[p].window_size.y, 32);
    }
    if (px > c->cfg.max_probe_pixels) return fail(c, LH_ERR_CAPACITY, "probe pixels exceed max_probe_pixels");
    return LH_OK;
}

}  // namespace

extern "C" {

uint32_t lh_version(void) { return kVersion; }

lh_status lh_create(const lh_config* config, lh_ctx** out) {
    if (!config || !out) return LH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lh_config cfg = *config;
    if (cfg.width == 0 || cfg.height == 0 || cfg.width > 16384 || cfg.height > 16384) return LH_ERR_INVALID_ARGUMENT;
    if (cfg.shadow_size == 0) cfg.shadow_size = 1024;
    if (cfg.shadow_size > 16384) return LH_ERR_INVALID_ARGUMENT;
    if (cfg.max_instances == 0) cfg.max_instances = MAX_INSTANCES;
    if (cfg.max_draws == 0) cfg.max_draws = MAX_OPAQUE_DRAWS;
    // draw slots (opaque + alpha) must fit the 24-bit visibility ID
    if ((uint64_t)cfg.max_draws * 2 > (1ull << 24)) return LH_ERR_INVALID_ARGUMENT;
    if (cfg.max_big_triangles == 0) cfg.max_big_triangles = 1u << 20;
    if (cfg.max_probes > kMaxViews - 5) return LH_ERR_INVALID_ARGUMENT;
    if (cfg.flags & ~LH_CONFIG_HDR_RGBA16F) return LH_ERR_INVALID_ARGUMENT;
    lh_ctx* c = new (std::nothrow) lh_ctx();
    if (!c) return LH_ERR_OUT_OF_MEMORY;
    c->cfg = cfg;
    c->device = cfg.device;
    c->tuning = lh_tuning{32u, 32u, 3.0f, LH_SCHEDULE_DEFAULT, 0u, 128u, {16u, 32u}, {128u, 64u}, 8u};
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    c->max_views = 5 + cfg.max_probes;
    c->sector_bytes = align_up(8 + 8 * (size_t)cfg.max_instances, 16);
    c->draw_bytes = align_up(8 + 16 * 2 * (size_t)cfg.max_draws, 16);
    const size_t W = cfg.width, H = cfg.height, S = cfg.shadow_size;
    uint8_t* frame_block = nullptr;  // kConstBytes of constants, then the Uniforms
    if (e == cudaSuccess) e = dalloc(c, &frame_block, kConstBytes + sizeof(Uniforms) * (1 + cfg.max_probes));
    if (e == cudaSuccess) {
        c->d_consts = reinterpret_cast<float*>(frame_block);
        c->d_uniforms = reinterpret_cast<Uniforms*>(frame_block + kConstBytes);
    }
    if (e == cudaSuccess) e = dalloc(c, &c->d_srgb, 256 * sizeof(float));
    if (e == cudaSuccess) e = dalloc(c, &c->d_misc, sizeof(MiscStorage));
    if (e == cudaSuccess) e = dalloc(c, &c->d_sectors, c->sector_bytes * c->max_views);
    if (e == cudaSuccess) e = dalloc(c, &c->d_refs, sizeof(MeshletReference) * 2 * (size_t)cfg.max_draws * c->max_views);
    if (e == cudaSuccess) e = dalloc(c, &c->d_rdraws, sizeof(RasterDraw) * 2 * (size_t)cfg.max_draws * c->max_views);
    if (e == cudaSuccess) e = dalloc(c, &c->d_lists, sizeof(uint32_t) * 3 * (size_t)cfg.max_draws * (1 + cfg.max_probes));
    // hierarchical depth: the main view, and the probes' total pixels in 64 x
    // 64 regions with room for each probe's partial regions
    c->hiz_words = align_up(((W + kHizRegion - 1) / kHizRegion) * ((H + kHizRegion - 1) / kHizRegion) * 65, 64) +
                   ((size_t)cfg.max_probe_pixels / (kHizRegion * kHizRegion) * 4 + 32 * (size_t)cfg.max_probes) * 65 +
                   64 * (size_t)cfg.max_probes;
    if (e == cudaSuccess) e = dalloc(c, &c->d_hiz, sizeof(uint32_t) * c->hiz_words);
    if (e == cudaSuccess) e = dalloc(c, &c->d_draws, c->draw_bytes * c->max_views);
    if (e == cudaSuccess) e = dalloc(c, &c->d_vis, W * H * 8);
    if (e == cudaSuccess) e = dalloc(c, &c->d_shadow, 4 * S * S * 4);
    if (e == cudaSuccess) e = dalloc(c, &c->d_hdr, W * H * hdr_pixel_bytes(c->cfg));
    if (e == cudaSuccess) e = dalloc(c, &c->d_probe_vis, (size_t)std::max(cfg.max_probe_pixels, 32u) * 8);
    if (e == cudaSuccess) e = dalloc(c, &c->d_big, sizeof(BigTri) * (size_t)cfg.max_big_triangles);
    if (e == cudaSuccess) e = dalloc(c, &c->d_big_base, sizeof(uint32_t) * (size_t)cfg.max_big_triangles);
    if (e == cudaSuccess) e = dalloc(c, &c->d_views, sizeof(ViewDev) * c->max_views);
    if (e == cudaSuccess) {
        float lut[256];
        for (int i = 0; i < 256; i++) {
            double v = i / 255.0;
            lut[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
        }
        e = cudaMemcpy(c->d_srgb, lut, sizeof(lut), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(c->d_misc, 0, sizeof(MiscStorage));
    if (e == cudaSuccess) c->vis_map_ok = encode_vis_map(c);
    c->staging_bytes = kConstBytes + sizeof(Uniforms) * (1 + cfg.max_probes);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaMallocHost(reinterpret_cast<void**>(&c->h_staging[i]), c->staging_bytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->staging_done[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->readback_done[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->resolved, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        lh_status st = e == cudaErrorMemoryAllocation ? LH_ERR_OUT_OF_MEMORY : LH_ERR_CUDA;
        free_all(c);
        delete c;
        return st;
    }
    *out = c;
    return LH_OK;
}

lh_status lh_set_scene(lh_ctx* c, const Instance* d_instances, uint32_t n, const lh_texture* textures,
                       uint32_t n_textures) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (n && !d_instances) return fail(c, LH_ERR_INVALID_ARGUMENT, "d_instances is NULL");
    if (((uintptr_t)d_instances & 15) != 0) return fail(c, LH_ERR_INVALID_ARGUMENT, "d_instances must be 16-byte aligned");
    if (n_textures && !textures) return fail(c, LH_ERR_INVALID_ARGUMENT, "textures is NULL");
    for (uint32_t i = 0; i < n_textures; i++)
        if (!textures[i].texels || !textures[i].width || !textures[i].height || (textures[i].texels & 3))
            return fail(c, LH_ERR_INVALID_ARGUMENT, "bad texture descriptor");
    cudaError_t e = cudaSuccess;
    drop_graph(c);
    c->instances = d_instances;
    c->n_instances = n;
    // total candidate meshlets bounds the look-back scratch
    // and whether any mesh is alpha clip (else the alpha-class launches are skipped)
    unsigned long long* d_sum = nullptr;
    e = cudaMalloc(&d_sum, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = launch_sum_meshlets(d_instances, n, d_sum, 0);
    unsigned long long sums[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(sums, d_sum, sizeof(sums), cudaMemcpyDeviceToHost);
    if (d_sum) cudaFree(d_sum);
    if (e != cudaSuccess) return cuda_fail(c, e, "scene meshlet count");
    c->scene_meshlets = sums[0];
    c->scene_alpha = (sums[1] & MESH_INFO_FLAGS_ALPHA_CLIP) != 0;
    // textures
    if (c->d_textures) {
        for (auto it = c->allocs.begin(); it != c->allocs.end(); ++it)
            if (it->p == c->d_textures) { cudaFree(it->p); c->allocs.erase(it); break; }
        c->d_textures = nullptr;
    }
    e = dalloc(c, &c->d_textures, sizeof(lh_texture) * std::max(1u, n_textures));
    if (e == cudaSuccess && n_textures)
        e = cudaMemcpy(c->d_textures, textures, sizeof(lh_texture) * n_textures, cudaMemcpyHostToDevice);
    c->n_textures = n_textures;
    // the kernels sample linear float4 texels: sRGB decoded through the LUT,
    // channels / 255 -- decoded here once instead of per sample
    for (void* old : {(void*)c->d_tex_linear, (void*)c->d_tex_linear_ptrs}) {
        if (!old) continue;
        for (auto it = c->allocs.begin(); it != c->allocs.end(); ++it)
            if (it->p == old) { cudaFree(it->p); c->allocs.erase(it); break; }
    }
    c->d_tex_linear = nullptr;
    c->d_tex_linear_ptrs = nullptr;
    {
        std::vector<size_t> offset(n_textures + 1, 0);
        for (uint32_t i = 0; i < n_textures; i++)
            offset[i + 1] = offset[i] + (size_t)textures[i].width * textures[i].height;
        if (e == cudaSuccess) e = dalloc(c, &c->d_tex_linear, sizeof(float4) * std::max<size_t>(1, offset[n_textures]));
        if (e == cudaSuccess) e = dalloc(c, &c->d_tex_linear_ptrs, sizeof(float4*) * std::max(1u, n_textures));
        std::vector<const float4*> ptrs(n_textures);
        c->tex_offset = offset;
        c->tex_size.assign(2 * (size_t)n_textures, 0u);
        for (uint32_t i = 0; i < n_textures; i++) {
            c->tex_size[2 * i] = textures[i].width;
            c->tex_size[2 * i + 1] = textures[i].height;
        }
        for (uint32_t i = 0; i < n_textures && e == cudaSuccess; i++) {
            ptrs[i] = c->d_tex_linear + offset[i];
            e = launch_linearize_texture(reinterpret_cast<const uchar4*>(textures[i].texels), c->d_tex_linear + offset[i],
                                         offset[i + 1] - offset[i], textures[i].srgb, c->d_srgb, 0);
        }
        if (e == cudaSuccess && n_textures)
            e = cudaMemcpy(c->d_tex_linear_ptrs, ptrs.data(), sizeof(float4*) * n_textures, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    // per-frame scratch
    if (c->d_reset) {
        for (auto it = c->allocs.begin(); it != c->allocs.end(); ++it)
            if (it->p == c->d_reset) { cudaFree(it->p); c->allocs.erase(it); break; }
        c->d_reset = nullptr;
    }
    c->reset_bytes = reset_bytes_for(c);
    if (e == cudaSuccess) e = dalloc(c, &c->d_reset, c->reset_bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "scene buffers");
    return prepare_views(c, nullptr, 0);
}

static lh_status frame_impl(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes, void* stream,
                            lh_frame_out* out, bool batched);
namespace {
lh_status frame_graph_impl(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes,
                           const GraphBackward* bw, void* stream, lh_frame_out* out, bool until_resolve = false);
}  // namespace

lh_status lh_frame(lh_ctx* c, const Uniforms* u, void* stream, lh_frame_out* out) {
    return frame_impl(c, u, nullptr, 0, stream, out, false);
}

lh_status lh_frame_readback(lh_ctx* c, const Uniforms* u, void* host_hdr, void* stream, lh_frame_out* out) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!host_hdr) return fail(c, LH_ERR_INVALID_ARGUMENT, "host_hdr is NULL");
    // replayed from the context's graph (up to the resolve) unless stage
    // timing is on, which needs the launches
    st = c->profiling ? frame_impl(c, u, nullptr, 0, stream, out, false)
                      : frame_graph_impl(c, u, nullptr, 0, nullptr, stream, out, true);
    if (st != LH_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t k = c->readbacks & 1u;
    const size_t bytes = (size_t)c->cfg.width * c->cfg.height * hdr_pixel_bytes(c->cfg);
    cudaError_t e = cudaEventRecord(c->resolved, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->resolved, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_hdr, c->d_hdr, bytes, cudaMemcpyDeviceToHost, c->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->readback_done[k], c->copy_stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "readback");
    c->readbacks++;
    // the previous call's image has landed once this returns
    if (c->readbacks > 1 && (e = cudaEventSynchronize(c->readback_done[k ^ 1u])) != cudaSuccess)
        return cuda_fail(c, e, "readback wait");
    return LH_OK;
}

lh_status lh_readback_wait(lh_ctx* c) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!c->readbacks) return LH_OK;
    cudaError_t e = cudaEventSynchronize(c->readback_done[(c->readbacks - 1) & 1u]);
    return e == cudaSuccess ? LH_OK : cuda_fail(c, e, "readback wait");
}

lh_status lh_frame_batched(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes, void* stream,
                           lh_frame_out* out) {
    return frame_impl(c, u, probes, n_probes, stream, out, true);
}

static lh_status frame_impl(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes, void* stream,
                            lh_frame_out* out, bool batched) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!u) return fail(c, LH_ERR_INVALID_ARGUMENT, "uniforms is NULL");
    if (!c->d_reset) return fail(c, LH_ERR_NO_SCENE, "lh_set_scene was not called");
    if (u->window_size.x != c->cfg.width || u->window_size.y != c->cfg.height)
        return fail(c, LH_ERR_INVALID_ARGUMENT, "uniforms.window_size differs from the context's size");
    if ((st = validate_probes(c, probes, n_probes)) != LH_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    bool same_views = n_probes == c->n_probes_last;
    if (same_views && n_probes) {
        for (uint32_t p = 0; p < n_probes && same_views; p++)
            same_views = probes[p].window_size.x == c->h_views[1 + p].width &&
                         probes[p].window_size.y == c->h_views[1 + p].height;
    }
    if (!same_views) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(c, e, "stream sync");
        if ((st = prepare_views(c, probes, n_probes)) != LH_OK) return st;
    }
    uint32_t n_inst = std::min(u->num_instances, c->n_instances);
    if (n_probes == 0 && frame_schedule(c, false) != LH_SCHEDULE_PERSISTENT) {
        // one main view: its uniforms ride on the clear launch
        const FrameStart start = make_frame_start(c, u);
        if ((st = enqueue_frame(c, n_probes, n_inst, batched, s, &start)) != LH_OK) return st;
    } else {
        if ((st = upload_frame_constants(c, u, probes, n_probes, s)) != LH_OK) return st;
        if ((st = enqueue_frame(c, n_probes, n_inst, batched, s)) != LH_OK) return st;
    }
    c->last_stream = s;
    if (out) fill_out(c, out);
    return LH_OK;
}

namespace {

// Batched frame replayed from a captured CUDA graph; with `bw` the resolve
// adjoint is captured into the same graph after the frame.
// `until_resolve` (plain frames only): the graph holds the frame up to the
// resolve, which is launched after it once the last pipelined readback of
// the image has landed -- so that readback overlaps the graph's culls and
// rasterisation instead of holding the whole graph back.
lh_status frame_graph_impl(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes,
                           const GraphBackward* bw, void* stream, lh_frame_out* out, bool until_resolve) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!u) return fail(c, LH_ERR_INVALID_ARGUMENT, "uniforms is NULL");
    if (!c->d_reset) return fail(c, LH_ERR_NO_SCENE, "lh_set_scene was not called");
    if (u->window_size.x != c->cfg.width || u->window_size.y != c->cfg.height)
        return fail(c, LH_ERR_INVALID_ARGUMENT, "uniforms.window_size differs from the context's size");
    if ((st = validate_probes(c, probes, n_probes)) != LH_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t n_inst = std::min(u->num_instances, c->n_instances);
    bool same_views = n_probes == c->n_probes_last;
    for (uint32_t p = 0; p < n_probes && same_views; p++)
        same_views = probes[p].window_size.x == c->h_views[1 + p].width &&
                     probes[p].window_size.y == c->h_views[1 + p].height;
    cudaError_t e;
    if (!same_views) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(c, e, "stream sync");
        if ((st = prepare_views(c, probes, n_probes)) != LH_OK) return st;
        drop_graph(c);
    }
    const bool tuning_changed = std::memcmp(&c->graph_tuning, &c->tuning, sizeof(lh_tuning)) != 0;
    const GraphBackward none{};
    const GraphBackward& want = bw ? *bw : none;
    const bool backward_changed = std::memcmp(&c->graph_backward, &want, sizeof(GraphBackward)) != 0;
    // one main view with a frame-start launch: its uniforms ride on that
    // kernel node's parameters (no copy before the replay)
    const bool plain = n_probes == 0 && frame_schedule(c, false) != LH_SCHEDULE_PERSISTENT;
    if (until_resolve && (n_probes || bw)) return fail(c, LH_ERR_INVALID_ARGUMENT, "readback graph of a plain frame only");
    if (!c->graph_exec || c->graph_probes != n_probes || c->graph_instances != n_inst || tuning_changed ||
        backward_changed || c->graph_until_resolve != until_resolve) {
        drop_graph(c);
        if (!c->capture_stream) {
            e = cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_fail(c, e, "capture stream");
        }
        e = cudaStreamBeginCapture(c->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(c, e, "begin capture");
        c->capturing = true;
        if (plain) {
            const FrameStart start = make_frame_start(c, u);
            st = enqueue_frame(c, n_probes, n_inst, true, c->capture_stream, &start, !until_resolve);
        } else {
            st = enqueue_frame(c, n_probes, n_inst, true, c->capture_stream, nullptr, !until_resolve);
        }
        if (st == LH_OK && bw) {
            const FrameDev f = frame_dev(c, 5 + n_probes, n_inst);
            cudaError_t eb = launch_resolve_backward(f, c->cfg.width, c->cfg.height,
                                                     reinterpret_cast<const float4*>(bw->grad), bw->targets,
                                                     c->capture_stream);
            if (eb != cudaSuccess) st = cuda_fail(c, eb, "resolve backward");
        }
        c->capturing = false;
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(c->capture_stream, &g);
        if (st != LH_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
        e = cudaGraphInstantiate(&c->graph_exec, g, 0);
        if (e == cudaSuccess && plain) {
            // the frame-start kernel node, updated before every replay
            size_t n = 0;
            e = cudaGraphGetNodes(g, nullptr, &n);
            std::vector<cudaGraphNode_t> nodes(n);
            if (e == cudaSuccess && n) e = cudaGraphGetNodes(g, nodes.data(), &n);
            for (size_t i = 0; e == cudaSuccess && i < n && !c->graph_clear_node; i++)
                if (is_clear_targets_node(nodes[i])) c->graph_clear_node = nodes[i];
            if (e == cudaSuccess && !c->graph_clear_node) e = cudaErrorInvalidValue;
        }
        if (e == cudaSuccess && plain) {
            c->graph_template = g;
        } else {
            cudaGraphDestroy(g);
        }
        if (e != cudaSuccess) {
            drop_graph(c);
            return cuda_fail(c, e, "graph instantiate");
        }
        c->graph_probes = n_probes;
        c->graph_instances = n_inst;
        c->graph_tuning = c->tuning;
        c->graph_backward = want;
        c->graph_until_resolve = until_resolve;
    }
    if (plain) {
        e = set_clear_targets_node(c->graph_exec, c->graph_clear_node, frame_dev(c, 5, n_inst), c->sms,
                                   make_frame_start(c, u));
        if (e != cudaSuccess) return cuda_fail(c, e, "graph frame start");
    } else if ((st = upload_frame_constants(c, u, probes, n_probes, s)) != LH_OK) {
        return st;
    }
    if (until_resolve) {
        e = cudaGraphLaunch(c->graph_exec, s);
        if (e == cudaSuccess) e = wait_readback(c, s);
        if (e == cudaSuccess) {
            const FrameDev f = frame_dev(c, 5, n_inst);
            e = launch_resolve(f, c->cfg.width, c->cfg.height, c->vis_map_ok ? &c->vis_map : nullptr, s, c->sms);
        }
    } else {
        e = wait_readback(c, s);
        if (e == cudaSuccess) e = cudaGraphLaunch(c->graph_exec, s);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
    c->last_stream = s;
    if (out) fill_out(c, out);
    return LH_OK;
}

}  // namespace

lh_status lh_frame_graph(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes, void* stream,
                         lh_frame_out* out) {
    return frame_graph_impl(c, u, probes, n_probes, nullptr, stream, out);
}

lh_status lh_frame_graph_backward(lh_ctx* c, const Uniforms* u, const Uniforms* probes, uint32_t n_probes,
                                  uint64_t d_grad_hdr, const lh_grad_targets* targets, void* stream,
                                  lh_frame_out* out) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!d_grad_hdr || !targets) return fail(c, LH_ERR_INVALID_ARGUMENT, "null gradient or targets");
    if ((d_grad_hdr & 15) || (targets->instance_grads & 7) || (targets->texture_grads & 7) ||
        (targets->light_dir & 3) || (targets->light_color & 3))
        return fail(c, LH_ERR_INVALID_ARGUMENT, "misaligned gradient buffer");
    GraphBackward bw{};
    bw.grad = d_grad_hdr;
    bw.targets = *targets;
    return frame_graph_impl(c, u, probes, n_probes, &bw, stream, out);
}

lh_status lh_get_outputs(lh_ctx* c, lh_frame_out* out) {
    if (!c || !out) return LH_ERR_INVALID_ARGUMENT;
    fill_out(c, out);
    return LH_OK;
}

lh_status lh_read_status(lh_ctx* c, lh_device_status* out) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!out) return LH_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    cudaError_t e = cudaStreamSynchronize(c->last_stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "stream sync");
    if (!c->d_reset) return LH_OK;
    uint32_t words[kStWords];
    e = cudaMemcpy(words, c->d_reset, sizeof(words), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "status read");
    out->flags = words[kStFlags];
    out->big_triangles = words[kStBigPacked + 1] >> 8;  // high word of the packed u64: count << 8
    out->clipped_triangles = words[kStClipCount];
    out->fragments[0] = words[kStFragVis];
    out->fragments[1] = words[kStFragShadow];
    if (!c->h_views.empty() && c->tuning.occlusion_px) {
        uint32_t claim[kClaimWords];
        e = cudaMemcpy(claim, c->h_views[0].claim, sizeof(claim), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "status read");
        out->occlusion[0] = claim[kClaimOccluders];
        out->occlusion[1] = claim[kClaimSurvivorsOpaque];
        out->occlusion[2] = claim[kClaimSurvivorsAlpha];
    }
    out->n_views = c->n_views_last;
    for (uint32_t v = 0; v < c->n_views_last && v < 40; v++) {
        unsigned long long counter = 0;
        uint32_t draws[2] = {0, 0};
        e = cudaMemcpy(&counter, c->h_views[v].sector, 8, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(draws, c->h_views[v].draws, 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "status read");
        out->visible_instances[v] = (uint32_t)(counter >> 32);
        out->candidate_meshlets[v] = (uint32_t)counter;
        out->visible_opaque[v] = draws[0];
        out->visible_alpha_clip[v] = draws[1];
    }
    return LH_OK;
}

lh_status lh_resolve_backward(lh_ctx* c, uint64_t d_grad_hdr, const lh_grad_targets* targets, void* stream) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!d_grad_hdr || !targets) return fail(c, LH_ERR_INVALID_ARGUMENT, "null gradient or targets");
    if (!c->d_reset) return fail(c, LH_ERR_NO_SCENE, "lh_set_scene was not called");
    if ((d_grad_hdr & 15) || (targets->instance_grads & 7) || (targets->texture_grads & 7) ||
        (targets->light_dir & 3) || (targets->light_color & 3))
        return fail(c, LH_ERR_INVALID_ARGUMENT, "misaligned gradient buffer");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    FrameDev f = frame_dev(c, c->n_views_last, c->n_instances);
    cudaError_t e = launch_resolve_backward(f, c->cfg.width, c->cfg.height, reinterpret_cast<const float4*>(d_grad_hdr),
                                            *targets, s);
    if (e != cudaSuccess) return cuda_fail(c, e, "resolve backward");
    c->last_stream = s;
    return LH_OK;
}

lh_status lh_get_texture_linear(lh_ctx* c, uint32_t index, uint64_t* d_texels, uint32_t* width, uint32_t* height) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!d_texels) return fail(c, LH_ERR_INVALID_ARGUMENT, "null output");
    if (!c->d_reset) return fail(c, LH_ERR_NO_SCENE, "lh_set_scene was not called");
    if (index >= c->n_textures || c->tex_offset.size() != (size_t)c->n_textures + 1)
        return fail(c, LH_ERR_INVALID_ARGUMENT, "texture index out of range");
    *d_texels = (uint64_t)(uintptr_t)(c->d_tex_linear + c->tex_offset[index]);
    if (width) *width = c->tex_size[2 * (size_t)index];
    if (height) *height = c->tex_size[2 * (size_t)index + 1];
    return LH_OK;
}

lh_status lh_display_transform(lh_ctx* c, uint64_t d_lut, uint64_t d_out, void* stream) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!d_out || (d_out & 3) || (d_lut & 15)) return fail(c, LH_ERR_INVALID_ARGUMENT, "null or misaligned buffer");
    if (!c->d_reset) return fail(c, LH_ERR_NO_SCENE, "lh_set_scene was not called");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (!d_lut && !c->d_lut_standin) {
        // identity on the encoded cube: texel (x, y, z) holds (x, y, z) / 47
        std::vector<float4> lut(48 * 48 * 48);
        for (int z = 0; z < 48; z++)
            for (int y = 0; y < 48; y++)
                for (int x = 0; x < 48; x++)
                    lut[((size_t)z * 48 + y) * 48 + x] = make_float4(x / 47.0f, y / 47.0f, z / 47.0f, 1.0f);
        e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = dalloc(c, &c->d_lut_standin, lut.size() * sizeof(float4));
        if (e == cudaSuccess)
            e = cudaMemcpy(c->d_lut_standin, lut.data(), lut.size() * sizeof(float4), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "stand-in LUT");
    }
    const float4* lut = d_lut ? reinterpret_cast<const float4*>(d_lut) : c->d_lut_standin;
    FrameDev f = frame_dev(c, c->n_views_last, c->n_instances);
    e = launch_display_transform(f, c->cfg.width, c->cfg.height, lut, reinterpret_cast<uchar4*>(d_out), s);
    if (e != cudaSuccess) return cuda_fail(c, e, "display transform");
    c->last_stream = s;
    return LH_OK;
}

lh_status lh_set_profiling(lh_ctx* c, int enable) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (enable && !c->stage_ev[0]) {
        for (auto& ev : c->stage_ev) {
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return cuda_fail(c, e, "event create");
        }
    }
    c->profiling = enable != 0;
    return LH_OK;
}

lh_status lh_get_stage_times(lh_ctx* c, float* ms, uint32_t n) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!ms || !c->profiling) return fail(c, LH_ERR_INVALID_ARGUMENT, "profiling is off");
    cudaError_t e = cudaEventSynchronize(c->stage_ev[LH_N_STAGES]);
    for (uint32_t i = 0; i < n && i < LH_N_STAGES && e == cudaSuccess; i++)
        e = cudaEventElapsedTime(&ms[i], c->stage_ev[i], c->stage_ev[i + 1]);
    if (e != cudaSuccess) return cuda_fail(c, e, "stage times");
    return LH_OK;
}

lh_status lh_download(lh_ctx* c, void* dst, uint64_t src, size_t bytes) {
    lh_status st = check_ctx(c);
    if (st != LH_OK) return st;
    if (!dst || !src) return fail(c, LH_ERR_INVALID_ARGUMENT, "null pointer");
    cudaError_t e = cudaStreamSynchronize(c->last_stream);
    if (e == cudaSuccess) e = cudaMemcpy(dst, reinterpret_cast<const void*>(src), bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "download");
    return LH_OK;
}

const char* lh_last_error(lh_ctx* c) { return c ? c->err.c_str() : "null context"; }

void lh_destroy(lh_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->last_stream) cudaStreamSynchronize(c->last_stream);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    free_all(c);
    delete c;
}

lh_status lh_set_tuning(lh_ctx* c, const lh_tuning* t) {
    if (!c || !t) return LH_ERR_INVALID_ARGUMENT;
    if (t->small_px > 4096 || t->medium_px < t->small_px || !(t->cull_blocks_per_sm > 0.0f) ||
        t->cull_blocks_per_sm > 64.0f || t->schedule > LH_SCHEDULE_PER_VIEW || t->raster_batch > 64 ||
        t->occlusion_px > 65536)
        return LH_ERR_INVALID_ARGUMENT;
    auto pow2_in = [](uint32_t v, uint32_t lo, uint32_t hi) { return v >= lo && v <= hi && (v & (v - 1)) == 0; };
    for (int k = 0; k < 2; k++)
        if (!pow2_in(t->chunk_rows[k], 4, 32) || !pow2_in(t->chunk_cols[k], 32, 256)) return LH_ERR_INVALID_ARGUMENT;
    if (!pow2_in(t->backward_rows, 4, 16)) return LH_ERR_INVALID_ARGUMENT;
    c->tuning = *t;
    return LH_OK;
}

lh_status lh_get_tuning(lh_ctx* c, lh_tuning* t) {
    if (!c || !t) return LH_ERR_INVALID_ARGUMENT;
    *t = c->tuning;
    return LH_OK;
}

}  // extern "C"
