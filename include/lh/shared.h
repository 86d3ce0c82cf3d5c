/*
 * CPU <-> GPU data contract of the visibility pipeline.
 *
 * Every struct here keeps the field order and the byte layout of the
 * reference's shared header (src/shared_cpu_gpu.h:12-157) as the GLSL side
 * sees it through `layout(scalar)` buffer references
 * (src/shaders/common/buffer_references.glsl:1-67): vec3 is 12 bytes with
 * 4-byte alignment, mat3 is 36 bytes, mat4 is 64 bytes, all column major.
 * Scene buffers are linked by 64-bit addresses exactly as with buffer device
 * addresses in the reference; on the GPU these are raw CUDA device pointers,
 * in the CPU oracle they are host pointers.
 *
 * The header is plain C so that it can be used from C, C++ and CUDA.
 */
#ifndef LH_SHARED_H
#define LH_SHARED_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lh_vec2 { float x, y; } lh_vec2;
typedef struct lh_vec3 { float x, y, z; } lh_vec3;
typedef struct lh_vec4 { float x, y, z, w; } lh_vec4;
typedef struct lh_uvec2 { uint32_t x, y; } lh_uvec2;
/* Column-major, cols[c] is column c (glm / GLSL convention). */
typedef struct lh_mat3 { lh_vec3 cols[3]; } lh_mat3;
typedef struct lh_mat4 { lh_vec4 cols[4]; } lh_mat4;

/* shared_cpu_gpu.h:8-9 */
#define MESH_INFO_FLAGS_32_BIT_INDICES 1u
#define MESH_INFO_FLAGS_ALPHA_CLIP 2u
/* Extension of this build: positions are f32x3, normals f32x3 and uvs f32x2
 * instead of the reference's u16x3 / i8x3 / u16x2 quantized attributes.
 * Bits 0-1 keep their meaning. */
#define MESH_INFO_FLAGS_FP32_VERTICES 4u

/* shared_cpu_gpu.h:12-16 (VkDispatchIndirectCommand) */
typedef struct DispatchIndirectCommand {
    uint32_t x, y, z;
} DispatchIndirectCommand;

/* shared_cpu_gpu.h:18-34 */
typedef struct MeshInfo {
    uint64_t positions;
    uint64_t indices;
    uint64_t normals;
    uint64_t uvs;
    uint64_t micro_indices;
    uint64_t meshlets;
    uint16_t num_meshlets;
    uint8_t flags;
    lh_vec4 bounding_sphere;
    lh_vec2 texture_scale;
    lh_vec2 texture_offset;
    uint16_t base_color_texture_index;
    uint16_t metallic_roughness_texture_index;
    uint16_t normal_texture_index;
    lh_vec3 base_color_factor;
} MeshInfo;

/* shared_cpu_gpu.h:36-43 */
typedef struct MiscStorage {
    lh_mat4 shadow_matrices[4];
    lh_mat4 uv_space_shadow_matrices[4];
    lh_mat4 shadow_view_matrices[4];
    float shadow_sphere_radii[4];
    uint32_t min_depth;
    uint32_t max_depth;
} MiscStorage;

/* shared_cpu_gpu.h:46-51 */
#define UNIFORMS_DEBUG_OFF 0
#define UNIFORMS_DEBUG_CASCADES 1
#define UNIFORMS_DEBUG_TRIANGLE_INDEX 2
#define UNIFORMS_DEBUG_INSTANCE_INDEX 3
#define UNIFORMS_DEBUG_SHADER_CLOCK 4
#define UNIFORMS_DEBUG_NORMALS 5

/* shared_cpu_gpu.h:53-76.  `debug_shadowmaps` is a GLSL bool, which is
 * 4 bytes in scalar layout; it is declared as uint32_t here. */
typedef struct Uniforms {
    lh_mat4 combined_perspective_view;
    lh_mat4 inv_perspective_view;
    lh_mat4 view;
    lh_mat4 initial_view;
    lh_mat4 perspective;
    lh_mat4 perspective_inverse;
    lh_mat4 view_inverse;
    uint64_t meshlet_references;
    uint64_t instances;
    uint64_t draw_calls;
    uint64_t misc_storage;
    uint64_t num_meshlets_prefix_sum;
    uint64_t dispatches;
    lh_vec3 camera_pos;
    lh_vec3 sun_dir;
    lh_vec3 sun_intensity;
    uint32_t num_instances;
    lh_uvec2 window_size;
    float shadow_cam_distance;
    float cascade_split_pow;
    int32_t debug;
    uint32_t debug_shadowmaps;
} Uniforms;

/* shared_cpu_gpu.h:79-84 (VkDrawIndirectCommand) */
typedef struct DrawIndirectCommand {
    uint32_t vertexCount;
    uint32_t instanceCount;
    uint32_t firstVertex;
    uint32_t firstInstance;
} DrawIndirectCommand;

/* shared_cpu_gpu.h:86-99 */
typedef struct Instance {
    lh_mat4 transform;
    uint64_t mesh_info_address;
    lh_mat3 normal_transform;
} Instance;

/* shared_cpu_gpu.h:119-127 (compile-time capacities in the reference; this
 * build takes the capacities at run time and keeps these as defaults). */
#define MAX_OPAQUE_DRAWS 200000u
#define MAX_ALPHA_CLIP_DRAWS 200000u
#define ALPHA_CLIP_DRAWS_OFFSET MAX_OPAQUE_DRAWS
#define MESHLET_INDICES_BUFFER_SECTION_OFFSET (ALPHA_CLIP_DRAWS_OFFSET + MAX_ALPHA_CLIP_DRAWS)
#define NEAR_PLANE 0.01f

/* shared_cpu_gpu.h:129-139 */
typedef struct Meshlet {
    lh_vec3 cone_apex;
    lh_vec3 cone_axis;
    float cone_cutoff;
    lh_vec4 bounding_sphere;
    uint32_t triangle_offset;
    uint32_t index_offset;
    uint8_t triangle_count;
    uint8_t index_count;
} Meshlet;

/* shared_cpu_gpu.h:142-145 */
typedef struct MeshletReference {
    uint32_t instance_index;
    uint16_t meshlet_index;
} MeshletReference;

/* shared_cpu_gpu.h:148-152 */
#define MAX_MESHLET_UNIQUE_VERTICES 64u
#define MAX_MESHLET_TRIANGLES 124u
#define MAX_MESHLET_VERTICES (MAX_MESHLET_TRIANGLES * 3u)
#define UNUSED_TEXTURE_INDEX 0xFFFFu

/* shared_cpu_gpu.h:154-157 */
typedef struct PrefixSumValue {
    uint32_t index;
    uint32_t sum;
} PrefixSumValue;

/* shared_cpu_gpu.h:159-166.  A prefix-sum sector is
 *   { uint64_t counter; PrefixSumValue values[capacity]; }
 * with counter = (number of entries << 32) | inclusive total
 * (src/shaders/common/prefix_sum.glsl:6-9,17-30). */
#define MAX_INSTANCES 1024u
#define PREFIX_SUM_BUFFER_SECTOR_SIZE (MAX_INSTANCES * 8u + 8u)
#define PER_INSTANCE_DISPATCH 0u
#define PER_SHADOW_INSTANCE_DISPATCH 1u
#define PER_MESHLET_DISPATCH 2u

/* Packed visibility ID, src/shaders/common/util.glsl:18-20:
 * triangle index in the top 8 bits, draw slot in the low 24. */
#define LH_PACK_ID(tri, slot) (((uint32_t)(tri) << 24) | (uint32_t)(slot))
#define LH_MAX_DRAW_SLOT ((1u << 24) - 1u)

#ifdef __cplusplus
}
#endif

/* Layout checks: byte offsets as the reference's scalar-layout GLSL sees them. */
#if defined(__cplusplus)
#include <cstddef>
#define LH_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#include <stddef.h>
#define LH_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif
LH_STATIC_ASSERT(sizeof(MeshInfo) == 104, "MeshInfo size");
LH_STATIC_ASSERT(offsetof(MeshInfo, num_meshlets) == 48, "MeshInfo.num_meshlets");
LH_STATIC_ASSERT(offsetof(MeshInfo, bounding_sphere) == 52, "MeshInfo.bounding_sphere");
LH_STATIC_ASSERT(offsetof(MeshInfo, texture_scale) == 68, "MeshInfo.texture_scale");
LH_STATIC_ASSERT(offsetof(MeshInfo, base_color_texture_index) == 84, "MeshInfo tex idx");
LH_STATIC_ASSERT(offsetof(MeshInfo, base_color_factor) == 92, "MeshInfo.base_color_factor");
LH_STATIC_ASSERT(sizeof(Instance) == 112, "Instance size");
LH_STATIC_ASSERT(offsetof(Instance, mesh_info_address) == 64, "Instance.mesh_info_address");
LH_STATIC_ASSERT(offsetof(Instance, normal_transform) == 72, "Instance.normal_transform");
LH_STATIC_ASSERT(sizeof(Meshlet) == 56, "Meshlet size");
LH_STATIC_ASSERT(offsetof(Meshlet, bounding_sphere) == 28, "Meshlet.bounding_sphere");
LH_STATIC_ASSERT(offsetof(Meshlet, triangle_offset) == 44, "Meshlet.triangle_offset");
LH_STATIC_ASSERT(offsetof(Meshlet, triangle_count) == 52, "Meshlet.triangle_count");
LH_STATIC_ASSERT(sizeof(MeshletReference) == 8, "MeshletReference size");
LH_STATIC_ASSERT(sizeof(Uniforms) == 560, "Uniforms size");
LH_STATIC_ASSERT(offsetof(Uniforms, meshlet_references) == 448, "Uniforms addresses");
LH_STATIC_ASSERT(offsetof(Uniforms, camera_pos) == 496, "Uniforms.camera_pos");
LH_STATIC_ASSERT(offsetof(Uniforms, num_instances) == 532, "Uniforms.num_instances");
LH_STATIC_ASSERT(offsetof(Uniforms, window_size) == 536, "Uniforms.window_size");
LH_STATIC_ASSERT(sizeof(MiscStorage) == 792, "MiscStorage size");
LH_STATIC_ASSERT(offsetof(MiscStorage, min_depth) == 784, "MiscStorage.min_depth");
LH_STATIC_ASSERT(sizeof(PrefixSumValue) == 8, "PrefixSumValue size");
LH_STATIC_ASSERT(sizeof(DrawIndirectCommand) == 16, "DrawIndirectCommand size");

#endif /* LH_SHARED_H */
