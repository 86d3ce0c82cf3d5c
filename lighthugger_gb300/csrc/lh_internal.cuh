// Device-visible frame description shared by the kernels and the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "lh/lh.h"

namespace lh {

constexpr uint32_t kMaxViews = 40;           // main + 4 cascades + up to 35 probes
constexpr uint32_t kInstTile = 256;          // instances per instance-cull tile
constexpr uint32_t kMlThreads = 256;         // threads per meshlet-cull block
#ifndef LH_ML_ITEMS
#define LH_ML_ITEMS 2
#endif
constexpr uint32_t kMlItems = LH_ML_ITEMS;   // candidates per thread (striped; 1, 2, 4 or 8)
constexpr uint32_t kMlTile = kMlThreads * kMlItems;
constexpr uint32_t kSpinLimit = 1u << 22;    // bounded waits (with __nanosleep back-off)

// Look-back status word: [63:62] 0 = not ready, 1 = tile aggregate,
// 2 = inclusive prefix; [61:0] payload (field-wise additive counts).
constexpr uint64_t kStatAgg = 1ull << 62;
constexpr uint64_t kStatIncl = 2ull << 62;
constexpr uint64_t kPayloadMask = (1ull << 62) - 1;

enum ViewKind : uint32_t { kViewVisibility = 0, kViewShadow = 1 };

// What the raster needs of one visible meshlet, with the address arithmetic
// done: written by the meshlet cull at the meshlet's draw slot, beside its
// MeshletReference.  The raster then reaches the vertices in three dependent
// loads (this record -> index words -> positions) where the reference chain
// takes six (MeshletReference -> Instance -> MeshInfo -> Meshlet -> index
// words -> positions; src/shaders/rasterization.glsl:12-37 and
// util.glsl:3-20 walk that chain per vertex).
struct __align__(16) RasterDraw {
    uint64_t positions;  // MeshInfo.positions
    uint64_t indices;    // MeshInfo.indices + Meshlet.index_offset elements
    uint64_t micro;      // MeshInfo.micro_indices + Meshlet.triangle_offset
    uint32_t instance;   // MeshletReference.instance_index
    uint32_t bits;       // index_count | triangle_count << 8 | MeshInfo.flags << 16 | kDrawNoCentre | kDrawOccluder
    float sphere[4];     // world-space sphere holding every vertex of the meshlet (centre, radius)
};
static_assert(sizeof(RasterDraw) == 48, "RasterDraw layout");
// RasterDraw::bits: the meshlet is rasterised in the occluder pass (a
// visibility view with occlusion culling, opaque, large on screen).
constexpr uint32_t kDrawOccluder = 1u << 31;
constexpr uint32_t kDrawNoCentre = 1u << 30;  // the world sphere reaches no pixel centre of the view
constexpr uint32_t kNoCentreTestPixels = 512u * 512u;  // views up to this size test it (sphere_box.cuh)

// Per-view lists of the two-pass occlusion raster of visibility views
// (ViewDev::lists, 3 * max_draws words): draw slots of the occluders, then
// of the opaque and the alpha-clip meshlets that survive the hierarchical
// depth test.  Their counts are ViewDev::claim[kClaimOccluders ...].
enum RasterList : uint32_t { kListAll = 0, kListOccluders = 1, kListSurvivors = 2 };
enum ClaimWord : uint32_t {
    kClaimInstTiles = 0,
    kClaimMeshletTiles = 1,
    kClaimOccluders = 2,       // entries of the occluder list
    kClaimSurvivorsOpaque = 3,
    kClaimSurvivorsAlpha = 4,
    kClaimWords = 8
};
// Hierarchical depth of a visibility view (ViewDev::hiz): level 0 holds the
// minimum depth bits of every 8 x 8-pixel tile, level 1 of every 64 x 64
// region, over the pixels written by the occluder pass (0 where a pixel has
// no fragment: a tile with an empty pixel culls nothing).  Regions are
// hiz_rx x hiz_ry; level 0 is row major with hiz_rx * 8 tiles per row,
// level 1 follows it.
constexpr uint32_t kHizTile = 8, kHizRegion = 64;

struct ViewDev {
    uint32_t kind;
    uint32_t cascade;
    uint32_t width, height;
    const Uniforms* uniforms;   // perspective views: their own; cascades: the main view's
    uint8_t* sector;            // prefix sector: u64 counter + PrefixSumValue[max_instances]
    MeshletReference* refs;     // 2*max_draws
    RasterDraw* rdraws;         // 2*max_draws, at the same slots as refs
    uint8_t* draws;             // u32 num_opaque, u32 num_alpha_clip, DrawIndirectCommand[2*max_draws]
    void* target;               // u64 visibility or u32 depth
    uint64_t* inst_status;      // per-frame zeroed look-back words, instance cull
    uint64_t* ml_status;        // per-frame zeroed look-back words, meshlet cull
    uint32_t* claim;            // per-frame zeroed kClaimWords: tile claims, occlusion list counts
    uint32_t section_base;      // firstInstance offset of this view's reference section
    uint32_t ml_tile_cap;       // capacity of ml_status
    uint32_t* lists;            // visibility views: occluder / survivor draw-slot lists (3 * max_draws)
    uint32_t* hiz;              // visibility views with occlusion culling: hierarchical depth, else null
    uint32_t hiz_rx, hiz_ry;    // 64 x 64-pixel regions of the view
};

// Triangle handed to the chunked raster path: its set-up (orientation
// normalised, pixel bounds) and its pixel bounds, cut into chunks of
// FrameDev::chunk_shift.
struct BigTri {
    int32_t X0, Y0, X1, Y1, X2, Y2;
    float z0, s1, s2;
    uint32_t id;
    uint32_t view;
    uint32_t bias;
    int32_t px0, px1, py0, py1;
};
// Chunk of a big triangle (one warp): rows x columns of pixels, powers of
// two chosen per pass at run time (lh_tuning.chunk_rows / chunk_cols, by
// the autotuner; at most 32 x 256): FrameDev::chunk_shift holds their log2.

// Per-frame scratch words (zeroed at frame start; the raster words again
// before each raster pass).
enum StatusWord : uint32_t {
    kStFlags = 0,
    kStClipCount = 1,  // triangles clipped in the last raster pass (statistics)
    kStRasterClaim = 2,
    kStBigClaim = 3,
    kStReduceDone = 4,
    // word 5 is unused
    kStMlClaim = 6,    // meshlet-cull (view, tile) claims
    kStBarrier = 7,    // grid barrier of the persistent kernel
    kStBigPacked = 8,  // u64 (words 8-9): big-triangle count << 40 | chunk count
    kStRasterClaimAlpha = 10,  // raster claims of the alpha-clip class
    kStFragVis = 11,     // fragments written this frame, visibility views (statistics)
    kStFragShadow = 12,  // the same, shadow views
    kStWords = 16
};

struct FrameDev {
    const Instance* instances;
    uint32_t n_instances;
    uint32_t max_instances;
    uint32_t max_draws;
    uint32_t n_views;
    MiscStorage* misc;
    uint32_t* status;           // kStWords words
    const ViewDev* views;       // n_views
    BigTri* big;
    uint32_t* big_base;         // first chunk of each big triangle (ascending)
    uint32_t big_cap;
    const lh_texture* textures;
    uint32_t n_textures;
    const float4* const* tex_linear;  // per texture: its texels as linear float4 (see launch_linearize_texture)
    float* shadow_maps;
    uint32_t shadow_size;
    void* hdr;               // float4[H][W], or (hdr_half) RGBA16F as 4 x half
    uint32_t hdr_half;
    uint64_t* visibility;       // main view
    const Uniforms* uniforms;   // main view
    const float* frame_consts;  // [0] pow(0.5, split), [1] pow(0.75, split)
    const float* srgb_lut;      // 256 entries
    uint32_t occlusion_px;      // occluder threshold (projected sphere radius, pixels); 0: no occlusion culling
    uint32_t chunk_shift[2][2]; // [pass: visibility, shadow][log2 rows, log2 columns] of a big-triangle chunk
    uint32_t backward_rows;     // pixel rows of a resolve-adjoint tile: 4, 8 or 16
    uint32_t scene_alpha;       // some mesh of the scene is alpha clip (else no alpha-class launch)
};

// Launch `kernel` with programmatic stream serialisation: its blocks may
// become resident while the previous kernel of the stream drains, hiding the
// launch gap between the frame's kernels (the kernel must begin with
// pdl_enter()).  Build with LH_PDL=0 for plain launches.
#ifndef LH_PDL
#define LH_PDL 1
#endif
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = LH_PDL ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Launchers (stream ordered).  Each returns the CUDA error of its launch.
// What the first kernel of a frame writes before anything reads it, when
// the host hands it over as a kernel parameter instead of two copies and a
// memset: the main view's Uniforms and the two frame constants, and the
// per-frame scratch zeroed.
struct FrameStart {
    Uniforms u;
    float consts[2];
    Uniforms* d_uniforms;
    float* d_consts;
    uint4* reset;          // per-frame scratch, zeroed
    uint64_t reset_words;  // its size in uint4
};
// dst[i] = texel i of an RGBA8 texture as linear floats: RGB through the
// sRGB decode table when `srgb`, else / 255; alpha / 255 (correctly rounded
// divisions, the oracle's definition).
cudaError_t launch_linearize_texture(const uchar4* src, float4* dst, size_t n, uint32_t srgb, const float* lut,
                                     cudaStream_t s);
// `targets` false: only the frame start and the counters (the instance-cull
// launches clear the targets, each with `clear_blocks` blocks per view).
cudaError_t launch_clear_targets(const FrameDev& f, cudaStream_t s, int sms, const FrameStart* start = nullptr,
                                 bool targets = true);
bool is_clear_targets_node(cudaGraphNode_t node);
cudaError_t set_clear_targets_node(cudaGraphExec_t exec, cudaGraphNode_t node, const FrameDev& f, int sms,
                                   const FrameStart& start);
cudaError_t launch_cull_instances(const FrameDev& f, uint32_t view_begin, uint32_t n_views, cudaStream_t s,
                                  uint32_t clear_blocks = 0);
cudaError_t launch_cull_meshlets(const FrameDev& f, uint32_t view_begin, uint32_t n_views, uint32_t blocks,
                                 cudaStream_t s);
// Raster all views [view_begin, view_begin + n_views) of one kind (kViewVisibility
// or kViewShadow): the opaque and alpha-clip classes (clipping inline), then
// the band kernel.
// With f.occlusion_px set, the visibility raster runs in two passes: the
// occluders, the hierarchical depth of what they wrote, the depth test of
// every other visible meshlet's bounding sphere against it, then the
// survivors (results identical: a skipped meshlet could not have won any
// pixel's depth test).
cudaError_t launch_raster_kind(const FrameDev& f, uint32_t view_begin, uint32_t n_views, int kind, uint32_t small_px,
                               uint32_t medium_px, uint32_t raster_batch, cudaStream_t s, int sms);
cudaError_t launch_depth_reduce_fit(const FrameDev& f, cudaStream_t s, int sms);
// Clear + cull + raster of every view in one cooperative persistent launch.
cudaError_t launch_frame_persistent(const FrameDev& f, uint32_t n_persp, uint32_t small_px, uint32_t medium_px,
                                    uint32_t raster_batch,
                                    float blocks_per_sm, cudaStream_t s, int sms);
int persistent_blocks_per_sm();
// vis_map: 2D tensor map of the main visibility buffer (u64, box 128 x 1) for
// the TMA-staged resolve, or null for per-thread loads.
cudaError_t launch_resolve(const FrameDev& f, uint32_t width, uint32_t height, const CUtensorMap* vis_map,
                           cudaStream_t s, int sms);
cudaError_t launch_display_transform(const FrameDev& f, uint32_t width, uint32_t height, const float4* lut, uchar4* out,
                                     cudaStream_t s);
cudaError_t launch_resolve_backward(const FrameDev& f, uint32_t width, uint32_t height, const float4* grad,
                                    const lh_grad_targets& t, cudaStream_t s);
cudaError_t launch_sum_meshlets(const Instance* instances, uint32_t n, unsigned long long* out, cudaStream_t s);

}  // namespace lh
