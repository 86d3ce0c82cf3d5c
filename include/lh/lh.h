/*
 * C ABI of the GB300 visibility pipeline.
 *
 * This is the drop-in boundary that replaces the reference's per-frame
 * `render()` call (src/rendering.h:4-16, src/rendering.cpp:28-548) and the
 * Vulkan objects behind it.  The reference enters its GPU passes through one
 * 8-byte push constant holding the address of the `Uniforms` buffer
 * (src/shaders/common/bindings.glsl:23-30, src/rendering.cpp:56-61); every
 * scene buffer is then reached through device addresses stored in
 * `Instance` / `MeshInfo` (src/shared_cpu_gpu.h:18-34,86-99).  Here the
 * caller hands over the same `Instance` array (device pointer, records
 * linking to caller-owned MeshInfo / vertex / meshlet buffers by device
 * address) and one `Uniforms` struct per frame from host memory.
 *
 * Conventions:
 *  - Ownership: the caller owns the scene buffers (like the reference's VMA
 *    buffers); the context owns all scratch and outputs (prefix sectors,
 *    visible lists, draw commands, visibility buffer, shadow maps, HDR).
 *  - Errors: every entry point returns an lh_status; nothing aborts.
 *    Device-side problems (capacity overflow, an expired bounded wait, a
 *    malformed meshlet) are recorded in a status word read by lh_read_status.
 *  - Threading: one context per host thread; work is stream ordered.
 *  - `stream` arguments are CUDA streams (cudaStream_t) passed as void*;
 *    NULL is the legacy default stream.
 */
#ifndef LH_LH_H
#define LH_LH_H

#include <stddef.h>
#include <stdint.h>

#include "shared.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lh_status;
#define LH_OK 0
#define LH_ERR_INVALID_ARGUMENT 1
#define LH_ERR_CUDA 2
#define LH_ERR_OUT_OF_MEMORY 3
#define LH_ERR_CAPACITY 4
#define LH_ERR_TIMEOUT 5
#define LH_ERR_NO_SCENE 6
#define LH_ERR_UNSUPPORTED 7

/* Device status flags (lh_device_status.flags). */
#define LH_FLAG_INSTANCE_OVERFLOW 0x1u /* more visible instances than max_instances */
#define LH_FLAG_DRAW_OVERFLOW 0x2u     /* more visible meshlets than max_draws */
#define LH_FLAG_QUEUE_OVERFLOW 0x4u    /* raster big-triangle queue full: triangles dropped */
#define LH_FLAG_TIMEOUT 0x8u           /* a bounded device-side wait expired */
#define LH_FLAG_BAD_MESHLET 0x10u      /* micro index >= meshlet vertex count: triangle skipped */
#define LH_FLAG_NO_DEPTH 0x20u         /* every main-view pixel is sky: cascades are NaN */
#define LH_FLAG_SLOT_OVERFLOW 0x40u    /* a draw slot does not fit the 24-bit visibility ID */

/* Rasterisation rules shared by every raster kernel (and restated by the
 * CPU oracle).  Vertices are snapped to 1/256 pixel; a pixel is covered when
 * its centre is inside the triangle under the top-left rule; triangles with
 * a vertex outside |x|,|y| <= LH_GUARD_BAND * w or outside 0 <= z <= w are
 * clipped in clip space first. */
#define LH_SUBPIXEL_BITS 8
#define LH_GUARD_BAND 256.0f

/* Texture descriptor: RGBA8 texels, row major, repeat addressing, bilinear
 * filtering of level 0.  `texels` is a device address for lh_set_scene. */
typedef struct lh_texture {
    uint64_t texels;
    uint32_t width;
    uint32_t height;
    uint32_t srgb; /* 1: RGB channels are sRGB encoded (decoded before filtering) */
    uint32_t reserved;
} lh_texture;

typedef struct lh_config {
    uint32_t width;           /* main view, pixels */
    uint32_t height;
    uint32_t shadow_size;     /* edge of each of the 4 cascade maps (1024 in the reference) */
    uint32_t max_instances;   /* prefix-sector capacity (MAX_INSTANCES = 1024 in the reference) */
    uint32_t max_draws;       /* visible meshlets per class per view (MAX_OPAQUE_DRAWS) */
    uint32_t max_big_triangles; /* raster overflow queue; 0 = default */
    uint32_t max_probes;      /* probe views for lh_frame_batched; 0 = none */
    uint32_t max_probe_pixels; /* total pixels over all probe views */
    int32_t device;           /* CUDA device ordinal */
    uint32_t flags;           /* LH_CONFIG_* bits; others must be 0 */
} lh_config;

/* lh_config.flags: the HDR image in RGBA16F (4 x IEEE half, round to
 * nearest even; the reference's frame_resources.h:20 format) instead of
 * RGBA32F.  Half the bytes written and read back; the differentiable resolve
 * needs RGBA32F. */
#define LH_CONFIG_HDR_RGBA16F 1u

/* Device pointers to the context-owned results of the last frame. */
typedef struct lh_frame_out {
    uint64_t visibility;   /* u64[height][width]: (float bits of depth << 32) | packed ID; 0 = clear */
    uint64_t hdr;          /* float4[height][width] (or 4 x half with LH_CONFIG_HDR_RGBA16F): linear HDR radiance, alpha = 1 */
    uint64_t shadow_maps;  /* float[4][shadow_size][shadow_size]: cascade depth, clear 1.0 */
    uint64_t misc_storage; /* MiscStorage */
    uint64_t prefix_sums;  /* n_views prefix sectors of prefix_sector_bytes each */
    uint64_t meshlet_references; /* n_views sections of 2*max_draws MeshletReference */
    uint64_t draw_calls;   /* n_views sections: {u32 num_opaque, u32 num_alpha_clip, DrawIndirectCommand[2*max_draws]} */
    uint64_t probe_visibility; /* u64 visibility of all probe views, packed back to back */
    uint64_t prefix_sector_bytes;
    uint64_t draw_call_section_bytes;
    uint32_t width, height, shadow_size, max_instances, max_draws;
    uint32_t n_views;      /* 5 for lh_frame: main, cascade 0..3 */
    uint32_t n_probes;
    uint32_t reserved;
} lh_frame_out;

typedef struct lh_device_status {
    uint32_t flags;
    uint32_t n_views;
    uint32_t visible_instances[40];  /* per view: entries in the prefix sector */
    uint32_t candidate_meshlets[40]; /* per view: inclusive total of the sector */
    uint32_t visible_opaque[40];     /* per view: num_opaque */
    uint32_t visible_alpha_clip[40]; /* per view: num_alpha_clip */
    uint32_t big_triangles;          /* triangles sent to the tiled raster path */
    uint32_t clipped_triangles;      /* triangles clipped (last raster pass) */
    uint32_t fragments[2];           /* fragments written this frame (one 64-bit depth-test reduction
                                        each): [0] visibility views, [1] shadow views */
    uint32_t occlusion[3];           /* main view, two-pass occlusion raster: occluder meshlets, then the
                                        opaque and alpha-clip meshlets that survived the depth test (the
                                        rest of the visible ones were skipped); 0 without occlusion */
} lh_device_status;

typedef struct lh_ctx lh_ctx;

/* Library version, for load checks. */
uint32_t lh_version(void);

/* Create a context: allocates every scratch and output buffer from the
 * capacities in `config` (replaces Resources / InstanceResources,
 * src/frame_resources.h:7-93, src/main.cpp:442-532). */
lh_status lh_create(const lh_config* config, lh_ctx** out_ctx);

/* Bind the scene: `d_instances` is a device array of n Instance records whose
 * mesh_info_address fields are device addresses (src/main.cpp:433-440);
 * `textures` is a host array of descriptors with device texel addresses,
 * indexed by MeshInfo texture indices (replaces the bindless texture array,
 * src/shaders/common/bindings.glsl:7, src/descriptor_set.cpp:28-139).
 * Texels are read here, once, into a linear float copy owned by the context
 * (16 bytes per texel; sRGB decoded), as the reference uploads its images
 * once: call lh_set_scene again after changing texel data.  Instance,
 * MeshInfo and vertex data are read by every frame; whether any mesh is
 * alpha clip (MESH_INFO_FLAGS_ALPHA_CLIP) is recorded here, so call
 * lh_set_scene again after setting that flag on a mesh of a scene that had
 * none. */
lh_status lh_set_scene(lh_ctx* ctx, const Instance* d_instances, uint32_t n,
                       const lh_texture* textures, uint32_t n_textures);

/* One frame (src/rendering.cpp:79-474): instance cull + prefix sum, meshlet
 * cull, visibility raster, depth reduction, cascade fit, shadow cull +
 * raster, lighting resolve.  `host_uniforms` is read during the call;
 * the address fields in it are ignored (the context supplies its own
 * buffers).  Asynchronous with respect to the host. */
lh_status lh_frame(lh_ctx* ctx, const Uniforms* host_uniforms, void* stream,
                   lh_frame_out* out);

/* Batched form: main view, 4 cascades and n_probes probe views (each probe
 * described by its own Uniforms: matrices, camera and window_size).  Cull
 * and raster of all views run in one persistent launch. */
lh_status lh_frame_batched(lh_ctx* ctx, const Uniforms* host_uniforms,
                           const Uniforms* probe_uniforms, uint32_t n_probes,
                           void* stream, lh_frame_out* out);

/* Same frame as lh_frame_batched, replayed from a CUDA graph: the first call
 * (or a call with different probe sizes, tuning or scene) captures the
 * frame's launches into a graph on a private stream; every call copies the
 * per-frame uniforms on `stream` and launches the graph there.  With no
 * probes the default schedule is the per-stage one of lh_frame. */
lh_status lh_frame_graph(lh_ctx* ctx, const Uniforms* host_uniforms,
                         const Uniforms* probe_uniforms, uint32_t n_probes,
                         void* stream, lh_frame_out* out);

/* Gradient buffers of one mesh for lh_resolve_backward (device addresses;
 * any may be 0 to skip it).  Gradients are added to what is there. */
typedef struct lh_mesh_grads {
    uint64_t positions;         /* float[3] per vertex: d/d(position as the shader reads it) */
    uint64_t normals;           /* float[3] per vertex: d/d(raw normal) */
    uint64_t uvs;               /* float[2] per vertex: d/d(raw uv) */
    uint64_t base_color_factor; /* float[3]: d/d(MeshInfo.base_color_factor) */
} lh_mesh_grads;

typedef struct lh_grad_targets {
    uint64_t instance_grads; /* device array [n_instances] of device addresses of lh_mesh_grads (0 = skip) */
    uint64_t texture_grads;  /* device array [n_textures] of device addresses of float4[h][w]: d/d(linear texel) (0 = skip) */
    uint64_t light_dir;      /* float[3]: d/d(Uniforms.sun_dir) */
    uint64_t light_color;    /* float[3]: d/d(Uniforms.sun_intensity), the light colour */
} lh_grad_targets;

/* Adjoint of the lighting resolve of the last frame with visibility held
 * fixed (triangle IDs, face flip, cascade choice and shadow-map compare
 * results are the forward's; everything continuous is differentiated).
 * `d_grad_hdr` is the upstream gradient, float4[height][width] (alpha
 * ignored).  The forward quantities are recomputed per pixel from the
 * visibility buffer, not stored.  Normal-mapped materials are not
 * differentiated.  No counterpart in the reference. */
lh_status lh_resolve_backward(lh_ctx* ctx, uint64_t d_grad_hdr, const lh_grad_targets* targets, void* stream);

/* lh_frame_graph followed by lh_resolve_backward of that frame, both in one
 * captured CUDA graph (re-captured when the views, instance count, tuning,
 * gradient buffer or targets change).  No counterpart in the reference. */
lh_status lh_frame_graph_backward(lh_ctx* ctx, const Uniforms* uniforms, const Uniforms* probes, uint32_t n_probes,
                                  uint64_t d_grad_hdr, const lh_grad_targets* targets, void* stream,
                                  lh_frame_out* out);

/* Device address (float4[height][width], linear RGBA) of the context's copy
 * of texture `index`, the texels every frame, the alpha test and the adjoint
 * sample; made by lh_set_scene from the caller's RGBA8 texels (sRGB
 * decoded, / 255).  Writing float4 values there, stream ordered before a
 * frame, changes what the following frames sample until the next
 * lh_set_scene -- how a differentiable caller applies texel parameters whose
 * gradients lh_resolve_backward writes (lh_grad_targets.texture_grads).  The
 * reference samples its bindless images instead; no counterpart there. */
lh_status lh_get_texture_linear(lh_ctx* ctx, uint32_t index, uint64_t* d_texels, uint32_t* width,
                                uint32_t* height);

/* Display transform of the last frame's HDR image (display_transform.comp:
 * 5-81): the tony_mc_mapface encoding stimulus / (stimulus + 1) into a 48^3
 * LUT sampled trilinearly (clamp to edge) at texel centres, the cascade
 * overlay when Uniforms.debug_shadowmaps is set, and the sRGB transfer
 * function, rounded to RGBA8.  d_lut: float4[48][48][48] (x fastest, indexed
 * by the encoded r, g, b), or 0 for the built-in identity stand-in (the
 * reference's LUT asset is not part of its sources).  d_out: uchar4[h][w].
 * Stream ordered, after the frame on the same stream. */
lh_status lh_display_transform(lh_ctx* ctx, uint64_t d_lut, uint64_t d_out, void* stream);

/* Pointers to the context's result buffers (valid until lh_destroy). */
lh_status lh_get_outputs(lh_ctx* ctx, lh_frame_out* out);

/* Synchronise the context's last stream and read the device status. */
lh_status lh_read_status(lh_ctx* ctx, lh_device_status* out);

/* Launch-shape knobs of the raster and cull kernels (set by the autotuner,
 * lighthugger_gb300/autotune.py) and the launch schedule.  Results never
 * depend on them. */
#define LH_SCHEDULE_DEFAULT 0    /* per stage */
#define LH_SCHEDULE_PER_STAGE 1  /* one launch per stage, each over all views of a kind */
#define LH_SCHEDULE_PERSISTENT 2 /* cull + raster of all views in one cooperative launch */
#define LH_SCHEDULE_PER_VIEW 3   /* each view's cull and raster launched on its own (the reference's per-cascade loop) */
typedef struct lh_tuning {
    uint32_t small_px;        /* a lane rasterises triangles whose bbox has <= small_px pixels */
    uint32_t medium_px;       /* the warp rasterises up to medium_px; larger go to chunks (chunk_rows x
                                 chunk_cols pixels, one warp each) */
    float cull_blocks_per_sm; /* meshlet-cull blocks per SM (per-stage schedule); blocks per SM (persistent) */
    uint32_t schedule;        /* LH_SCHEDULE_* */
    uint32_t raster_batch;    /* meshlets a raster warp claims per atomic (0: 4 when the views hold more than
                                 256 meshlets per warp of the grid, else 1) */
    uint32_t occlusion_px;    /* two-pass occlusion raster of the visibility views: opaque meshlets whose
                                 bounding sphere projects to a radius above this many pixels are drawn
                                 first, the hierarchical depth of what they wrote is built, and every other
                                 meshlet whose sphere lies behind it is skipped (no counterpart in the
                                 reference; results identical).  0: one pass, no occlusion test */
    uint32_t chunk_rows[2];   /* pixel rows of a big-triangle chunk (one warp) in the visibility / shadow
                                 pass: 4, 8, 16 or 32 */
    uint32_t chunk_cols[2];   /* its columns: 32, 64, 128 or 256 */
    uint32_t backward_rows;   /* pixel rows of a resolve-adjoint tile (one warp per row): 4, 8 or 16 */
} lh_tuning;
/* lh_create's tuning: lane bin 32 pixels and no warp bin (medium_px 32),
 * occluders above 128 px, chunks of 16 x 128 (visibility) and 32 x 64
 * (shadow) pixels, adjoint tiles of 8 rows, 3 meshlet-cull blocks per SM
 * (as many as are resident at once). */

lh_status lh_set_tuning(lh_ctx* ctx, const lh_tuning* tuning);
lh_status lh_get_tuning(lh_ctx* ctx, lh_tuning* tuning);

/* Per-stage timing with CUDA events recorded on the frame's stream (the
 * replacement of the reference's Tracy GPU zones, src/rendering.cpp:41-42,
 * 140-492).  Stages: 0 frame start (uniforms, counters), 1 cull instances
 * (with the visibility targets' clear), 2 cull meshlets, 3 raster, 4 depth
 * reduce + cascade fit, 5 shadow instance cull (with the shadow maps'
 * clear), 6 shadow meshlet cull, 7 shadow raster, 8 resolve. */
#define LH_N_STAGES 9
lh_status lh_set_profiling(lh_ctx* ctx, int enable);
/* Milliseconds of each stage of the last profiled frame (synchronises). */
lh_status lh_get_stage_times(lh_ctx* ctx, float* ms, uint32_t n);

/* Instance cull + single-pass prefix sum of one view that allocates
 * nothing.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc -- an engine that owns all device memory under a
 * fixed budget, a frame loop that must not stall on an allocation (cudaMalloc
 * can synchronise the device), code recording into a stream capture.
 * Inputs: the device Instance array (16-byte aligned) and host Uniforms
 * (passed to the kernel by value).  Output: a caller-owned prefix sector
 * {u64 counter; PrefixSumValue[capacity]} in device memory, identical to
 * lh_frame's main-view sector.  `d_flags` (optional, device) receives
 * LH_FLAG_* bits.  The kernel's scratch is a fixed array inside the library
 * of about 33 KB per GPU, so n_instances is limited to 1,048,576
 * (LH_ERR_CAPACITY beyond).  A call outside stream capture looks up that
 * array's address on the current device; a call during capture reuses the
 * address found by the last call outside capture (LH_ERR_UNSUPPORTED if there
 * was none), so the first call on a device should come before any stream
 * capture.  All calls share the array, so calls that overlap on the GPU
 * race -- serialise them.  Every block ORs the flags it raises into d_flags
 * itself (LH_FLAG_TIMEOUT, LH_FLAG_INSTANCE_OVERFLOW); with more visible
 * instances than `capacity` the counter holds the true count and entries
 * stop at `capacity`. */
lh_status lh_cull_instances_noalloc(const Instance* d_instances, uint32_t n_instances,
                                    const Uniforms* host_uniforms, uint8_t* d_sector, uint32_t capacity,
                                    uint32_t* d_flags, void* stream);

/* Diagnostic: run one of the library's bounded device-side waits -- the
 * decoupled look-back of the culls (LH_WAIT_LOOKBACK), the grid barrier of
 * the persistent frame kernel (LH_WAIT_GRID_BARRIER) or the mbarrier wait of
 * the TMA-staged resolve (LH_WAIT_MBARRIER) -- in a one-block launch whose
 * condition is met at once (`satisfied` != 0) or never (a predecessor that
 * never publishes, a block that never arrives, an arrival that never comes),
 * polling at most `poll_limit` times (1 .. 2^22).  `d_words`: 8 device u64
 * words, zeroed by the call; once the stream has run it, word 3 (low 32
 * bits) holds LH_FLAG_TIMEOUT if the wait expired and word 4 the wait's
 * result (the look-back's exclusive prefix: 5 from its predecessor, or 0
 * when that never published; else 1 when the wait completed).  Checks the
 * failure path of the frame kernels without a fault or a hang.  No
 * counterpart in the reference. */
#define LH_WAIT_LOOKBACK 0u
#define LH_WAIT_GRID_BARRIER 1u
#define LH_WAIT_MBARRIER 2u
lh_status lh_check_bounded_wait(uint32_t which, uint32_t poll_limit, uint32_t satisfied, uint64_t* d_words,
                                void* stream);

/* Throughput probe of the raster's depth test (no counterpart in the
 * reference, whose depth test is fixed-function): `reps` passes of 64-bit
 * max reductions (red.relaxed.gpu.global.max.u64, no return) over the
 * n_words words at d_words -- each pass one reduction per word, to word i
 * (`scattered` 0: a warp covers 256 contiguous bytes) or to a pseudo-random
 * word (1: every lane its own cache line).  Time it with events on `stream`:
 * n_words * reps / seconds is the reductions-per-second ceiling the raster's
 * fragments are measured against.  The buffer's contents are overwritten. */
lh_status lh_probe_red_u64(uint64_t* d_words, uint64_t n_words, uint32_t scattered, uint32_t reps, void* stream);

/* The plain frame (as lh_frame) followed by a copy of the HDR image (width *
 * height pixels of 16 bytes, 8 with LH_CONFIG_HDR_RGBA16F) to `host_hdr`,
 * pipelined: the frame up to the resolve is replayed from the context's CUDA
 * graph, the resolve is launched once the previous call's copy has landed,
 * and the copy runs on a stream of the context after it -- so the next
 * frame's culling and rasterisation run while it lands.  Returns once both are
 * enqueued and the PREVIOUS call's copy has landed, so callers alternate two
 * host buffers (pinned for an asynchronous copy): after call i returns, the
 * buffer of call i - 1 holds its frame.  lh_readback_wait waits for the last
 * copy.  The reference presents its frame instead; no counterpart there. */
lh_status lh_frame_readback(lh_ctx* ctx, const Uniforms* host_uniforms, void* host_hdr, void* stream,
                            lh_frame_out* out);
lh_status lh_readback_wait(lh_ctx* ctx);

/* Synchronise the context's last stream and copy `bytes` from a device
 * address (e.g. a field of lh_frame_out) to host memory. */
lh_status lh_download(lh_ctx* ctx, void* host_dst, uint64_t device_src, size_t bytes);

/* Human-readable text of the last host-side error of this context. */
const char* lh_last_error(lh_ctx* ctx);

void lh_destroy(lh_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* LH_LH_H */
