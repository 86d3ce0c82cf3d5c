/*
 * CPU oracle of the visibility pipeline -- TEST INFRASTRUCTURE ONLY.
 *
 * A C++ restatement of the reference's GLSL passes (expenses/lighthugger,
 * src/shaders/) and of the Vulkan fixed-function rules they rely on
 * (rasterisation, depth test, bilinear and comparison sampling).  It is the
 * checker the CUDA path is compared against and the timed CPU baseline; the
 * product path never links, loads or calls it.
 *
 * Parity status: UNPINNED against the reference itself.  The reference is a
 * Vulkan renderer with no tests, golden vectors or CPU path, and it cannot be
 * built or run here (no Vulkan, glslc or graphics stack, empty submodules).
 * The oracle is pinned instead by hand-derived known-answer tests
 * (tests/test_oracle_known_answers.py) and by its float64 twin of the
 * resolve (lho_resolve_f64); its outputs on four seeded scenes are held
 * fixed by the golden digests of tests/golden/oracle_frames.json
 * (tests/test_golden.py).
 *
 * Evaluation-order contract (shared with the CUDA kernels so that integer,
 * visibility and depth results can be bit exact): every float operation is a
 * single IEEE-754 binary32 operation rounded to nearest, with no fused
 * multiply-add (built with -ffp-contract=off; kernels with --fmad=false);
 *   dot(a,b)      = (a.x*b.x + a.y*b.y) + a.z*b.z
 *   length(v)     = sqrt(dot(v,v));  normalize(v) = v / length(v) per component
 *   M*v (mat4)    = ((c0*v.x + c1*v.y) + c2*v.z) + c3*v.w per row
 *   mix(x,y,a)    = x*(1-a) + y*a
 * pow() is the only transcendental on the path (cascade split exponent on
 * the host in double; BRDF Schlick terms and sky exposure per pixel), so
 * HDR radiance is compared with a 2^-10 tolerance while culling,
 * visibility, depth and shadow maps compare bit for bit.
 */
#ifndef LH_ORACLE_H
#define LH_ORACLE_H

#include <stdint.h>

#include "../include/lh/lh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Stage mask for lho_frame. */
#define LHO_STAGE_CULL 1u
#define LHO_STAGE_RASTER 2u
#define LHO_STAGE_DEPTH 4u
#define LHO_STAGE_SHADOW 8u
#define LHO_STAGE_RESOLVE 16u
#define LHO_STAGE_ALL 31u

typedef struct lho_frame_desc {
    const Instance* instances;   /* host records, host mesh_info_address */
    uint32_t n_instances;
    const lh_texture* textures;  /* host texel addresses */
    uint32_t n_textures;
    const Uniforms* uniforms;    /* window_size = main view size */
    uint32_t shadow_size;
    uint32_t max_instances;
    uint32_t max_draws;
    int32_t threads;             /* <= 0: all hardware threads */
    uint32_t stages;
    /* optional (may be null; entries may be null): per texture, width*height
     * linear RGBA floats sampled in place of its RGBA8 texels -- the values
     * the kernels sample (sRGB decoded, / 255), so that the float64 resolve
     * can be differentiated with respect to a texel */
    const float* const* texture_linear;
} lho_frame_desc;

/* All buffers are caller allocated, in the layouts lh_frame_out documents:
 *   prefix_sums: 5 sectors of 8 + 8*max_instances bytes (main, cascade 0..3)
 *   meshlet_references: 5 sections of 2*max_draws MeshletReference
 *   draw_calls: 5 sections of 8 + 16*2*max_draws bytes
 *   visibility: width*height u64;  shadow_maps: 4*S*S float;  hdr: W*H*4 float */
typedef struct lho_frame_out {
    uint8_t* prefix_sums;
    MeshletReference* meshlet_references;
    uint8_t* draw_calls;
    uint64_t* visibility;
    float* shadow_maps;
    MiscStorage* misc;
    float* hdr;
    double stage_ms[8]; /* cull, raster, depth+fit, shadow cull, shadow raster, resolve, total, threads */
    uint32_t flags;     /* LH_FLAG_* */
    uint32_t reserved;
    /* raster statistics, [0..7] visibility views, [8..15] shadow views:
     * triangles set up, fragments covered, bbox <= 4 px, <= 64, <= 4096,
     * > 4096, clipped, max fragments of one meshlet */
    uint64_t stats[16];
} lho_frame_out;

int lho_frame(const lho_frame_desc* desc, lho_frame_out* out);

/* Rasterise a single clip-space triangle into a u64 visibility target with
 * the pipeline's rules (known-answer tests).  kind 0: visibility (cull back
 * faces, keep max of (depth bits << 32 | id)); kind 1: shadow depth (cull
 * front faces, keep min depth bits in the low 32 bits of each u64). */
int lho_raster_triangle(const float clip[12], uint32_t id, uint32_t kind, uint32_t width, uint32_t height,
                        uint64_t* target);

/* The same for an alpha-clip draw: double sided, each fragment kept only
 * when the alpha of `texture` (host texels), sampled bilinearly with repeat
 * addressing at the perspective-correct uv of the pixel centre (per-vertex
 * uvs in `uv[6]`), is not below 0.5. */
int lho_raster_triangle_alpha(const float clip[12], const float uv[6], const lh_texture* texture, uint32_t id,
                              uint32_t kind, uint32_t width, uint32_t height, uint64_t* target);

/* Display transform (display_transform.comp:5-81) of a float RGBA HDR image
 * into RGBA8: tony_mc_mapface encoding into a 48^3 LUT (float4, x fastest;
 * null = the identity stand-in), the cascade overlay when debug_shadowmaps,
 * sRGB transfer function, round to nearest. */
int lho_display_transform(const float* hdr, uint32_t width, uint32_t height, const float* lut, const float* shadow_maps,
                          uint32_t shadow_size, uint32_t debug_shadowmaps, uint8_t* out);

/* Forward resolve of one frame in float64 (the FP64 reference for error
 * statements); same inputs as lho_frame with visibility and shadow maps
 * already filled in `out`. */
int lho_resolve_f64(const lho_frame_desc* desc, const lho_frame_out* in, double* hdr64);

/* The same for the n pixels listed in xy (x, y pairs); hdr64 receives 4
 * doubles per listed pixel. */
int lho_resolve_f64_pixels(const lho_frame_desc* desc, const lho_frame_out* in, const uint32_t* xy, uint32_t n,
                           double* hdr64);

#ifdef __cplusplus
}
#endif

#endif
