/*
 * Seeded synthetic scenes for the visibility pipeline, and the host-side
 * uniform math the reference does per frame.
 *
 * The reference loads one glTF scene and meshletises it with meshoptimizer
 * (src/resources/mesh_loading.cpp:241-738, src/resources/meshlets.cpp:3-140).
 * Neither the scene nor meshoptimizer is available, so this module builds
 * procedural meshes, meshletises them itself (<= 64 vertices, <= 124
 * triangles, u8 micro-indices, 4-byte aligned triangle offsets as at
 * meshlets.cpp:62-64), computes its own normal cones and bounding spheres,
 * and lays everything out exactly as the reference's buffers: MeshInfo,
 * Meshlet, index and micro-index arrays, Instance records.
 *
 * A scene exists twice: a host copy whose address fields hold host pointers
 * (what the CPU oracle walks) and, after lh_scene_upload, a device copy whose
 * address fields hold CUDA device pointers (what lh_set_scene takes).
 */
#ifndef LH_SCENE_H
#define LH_SCENE_H

#include "lh.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lh_scene lh_scene;

/* Overrides of a config's defaults; zero fields keep the default. */
typedef struct lh_scene_params {
    uint32_t width, height;     /* main view */
    uint32_t n_instances;
    uint32_t n_probes;          /* probe views (config 3 default 32) */
    float detail;               /* multiplies mesh triangle counts (0 = 1.0) */
    uint32_t quantized;         /* 1: u16 positions / i8 normals / u16 uvs (reference formats) */
    uint32_t reference_normal_transform; /* 1: normal_transform = mat3(inverse(M)) as the reference's constructor */
    uint32_t alpha_clip_materials; /* 1: odd materials are alpha clipped */
    uint32_t reserved[4];
} lh_scene_params;

typedef struct lh_scene_desc {
    uint32_t config_id;
    uint32_t n_instances;
    uint32_t n_meshes;
    uint32_t n_textures;
    uint32_t n_probes;
    uint32_t width, height;
    uint32_t shadow_size;       /* config's cascade size */
    uint64_t total_meshlets;    /* sum over instances of num_meshlets */
    uint64_t total_triangles;   /* sum over instances of mesh triangles */
    uint64_t seed;
    const Instance* host_instances;   /* mesh_info_address = host MeshInfo address */
    const lh_texture* host_textures;  /* texels = host address */
    const Instance* device_instances; /* NULL before lh_scene_upload */
    const lh_texture* device_textures; /* host array, texels = device address */
    Uniforms uniforms;                /* main camera, addresses zero */
    const Uniforms* probes;           /* n_probes camera uniforms */
    uint64_t device_bytes;            /* bytes uploaded */
} lh_scene_desc;

/* Build config `config_id` (1..5) with `seed`; params may be NULL. */
lh_status lh_scene_create(uint32_t config_id, uint64_t seed, const lh_scene_params* params,
                          lh_scene** out);
/* A scene of one caller mesh (a triangle list) drawn by n_instances
 * instances: meshletised like the synthetic meshes (fp32 attributes, 32-bit
 * indices), one untextured material, the camera `uniforms` (address fields
 * ignored; num_instances set).  positions: float[3] per vertex, finite;
 * normals: float[3] per vertex or NULL (area-weighted vertex normals); uvs:
 * float[2] per vertex or NULL (zero); indices: 3 per triangle, each below
 * n_vertices; transforms: one lh_mat4 (column major) per instance. */
lh_status lh_scene_from_mesh(const float* positions, const float* normals, const float* uvs, uint32_t n_vertices,
                             const uint32_t* indices, uint32_t n_triangles, const lh_mat4* transforms,
                             uint32_t n_instances, const Uniforms* uniforms, lh_scene** out);
lh_status lh_scene_describe(const lh_scene* scene, lh_scene_desc* out);
/* Copy meshes, instances and textures to `device`; patch device addresses. */
lh_status lh_scene_upload(lh_scene* scene, int device);
void lh_scene_destroy(lh_scene* scene);

/* One MeshInfo record of a scene (one per mesh x material pair). */
typedef struct lh_scene_mesh {
    const MeshInfo* host_info; /* host record (host addresses inside) */
    uint64_t device_info;      /* device address of the record; 0 before lh_scene_upload */
    uint64_t device_positions, device_normals, device_uvs; /* the record's device buffers */
    uint32_t mesh;             /* index of the vertex buffers (records of one mesh share them) */
    uint32_t vertices;
    uint32_t triangles;
    uint32_t flags;
} lh_scene_mesh;

uint32_t lh_scene_mesh_count(const lh_scene* scene);
lh_status lh_scene_mesh_get(const lh_scene* scene, uint32_t index, lh_scene_mesh* out);
/* MeshInfo record index of every instance (out: n_instances entries). */
lh_status lh_scene_instance_records(const lh_scene* scene, uint32_t* out);

/* Scene dumps: a flat binary file of a scene's host copy -- the meshes'
 * vertex, index, micro-index and Meshlet buffers, the MeshInfo and Instance
 * records in their shared layouts (address fields stored as zero and
 * relinked at load), the texel arrays, the camera and probe Uniforms -- so
 * that a frame can be replayed from a file (by the oracle, or on the GPU
 * after lh_scene_upload).  The file is in the host's byte order.
 * lh_scene_load returns LH_ERR_INVALID_ARGUMENT for a file that is not a
 * complete dump (wrong magic or version, truncated, an index out of range)
 * and LH_ERR_UNSUPPORTED when the file cannot be opened; lh_scene_save
 * returns LH_ERR_UNSUPPORTED when it cannot be written. */
lh_status lh_scene_save(const lh_scene* scene, const char* path);
lh_status lh_scene_load(const char* path, lh_scene** out);

/* Camera as the reference's CameraParams (src/input.h:18-49) plus the
 * window; fov in degrees. */
typedef struct lh_camera {
    lh_vec3 position;
    float yaw, pitch, fov_degrees;
    float sun_latitude, sun_longitude;
    uint32_t width, height;
    float shadow_cam_distance; /* 1024 in the reference */
    float cascade_split_pow;   /* 3 in the reference */
    uint32_t num_instances;
} lh_camera;

/* Per-frame uniform math of src/main.cpp:734-760: lookAt view,
 * infinite reverse-Z perspective (src/projection.h:3-20), their product
 * and inverses, sun direction (src/input.h:43-49). */
lh_status lh_make_uniforms(const lh_camera* camera, Uniforms* out);

#ifdef __cplusplus
}
#endif

#endif
