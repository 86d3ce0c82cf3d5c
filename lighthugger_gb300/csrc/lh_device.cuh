// Device-side building blocks of the visibility pipeline: GLSL-ordered float
// math, scene access through device addresses, the culling tests, the
// rasterisation rules and the samplers.
//
// Every kernel including this file is compiled with --fmad=false and IEEE
// division / square root, so each float operation below rounds on its own;
// the evaluation orders are the ones the CPU oracle states (dot =
// (x*x' + y*y') + z*z', mat4*vec4 = ((c0*x + c1*y) + c2*z) + c3*w, ...),
// which makes culling, visibility IDs, depth and shadow maps bit exact.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

#include "int_float.cuh"
#include "lh/lh.h"

namespace lh {

// Programmatic dependent launch.  A frame kernel launched by launch_pdl may
// be scheduled while the kernel before it in the stream is still finishing;
// its first statement waits (griddepcontrol.wait) until that kernel has
// completed and its writes are visible, so nothing is read or written
// early, and then lets the next kernel of the stream begin launching.  In a
// kernel launched without the attribute both instructions return at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ------------------------------------------------------------------ vectors
struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float length(f3 v) { return sqrtf(dot(v, v)); }
__device__ __forceinline__ f3 normalize(f3 v) { float l = length(v); return {v.x / l, v.y / l, v.z / l}; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ f3 ld3(const lh_vec3& v) { return {v.x, v.y, v.z}; }

// mat4 * vec4 with the column-major reference layout.
__device__ __forceinline__ f4 mul(const lh_mat4& m, f4 v) {
    const lh_vec4 &c0 = m.cols[0], &c1 = m.cols[1], &c2 = m.cols[2], &c3 = m.cols[3];
    return {((c0.x * v.x + c1.x * v.y) + c2.x * v.z) + c3.x * v.w,
            ((c0.y * v.x + c1.y * v.y) + c2.y * v.z) + c3.y * v.w,
            ((c0.z * v.x + c1.z * v.y) + c2.z * v.z) + c3.z * v.w,
            ((c0.w * v.x + c1.w * v.y) + c2.w * v.z) + c3.w * v.w};
}
__device__ __forceinline__ f3 mul3(const lh_mat3& m, f3 v) {
    const lh_vec3 &c0 = m.cols[0], &c1 = m.cols[1], &c2 = m.cols[2];
    return {(c0.x * v.x + c1.x * v.y) + c2.x * v.z, (c0.y * v.x + c1.y * v.y) + c2.y * v.z,
            (c0.z * v.x + c1.z * v.y) + c2.z * v.z};
}
// max/min with the std::max / std::min conventions the oracle uses
// (the first argument is kept when the comparison is false).
__device__ __forceinline__ float gmax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float gmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }

// Repeat addressing of texel coordinate i into [0, n): the floor of a
// sample coordinate below 1e9 in magnitude, so 32 bits hold it.
__device__ __forceinline__ int32_t wrap_texel(int32_t i, int32_t n) {
    if ((n & (n - 1)) == 0) return i & (n - 1);
    const int32_t r = i % n;
    return r < 0 ? r + n : r;
}

// ------------------------------------------------------------------ scene access
__device__ __forceinline__ const MeshInfo* mesh_info_of(const Instance* inst) {
    return reinterpret_cast<const MeshInfo*>(inst->mesh_info_address);
}
__device__ __forceinline__ uint32_t load_index(const MeshInfo* mi, uint32_t flags, uint32_t vertex_id) {
    if (flags & MESH_INFO_FLAGS_32_BIT_INDICES) return __ldg(reinterpret_cast<const uint32_t*>(mi->indices) + vertex_id);
    return __ldg(reinterpret_cast<const uint16_t*>(mi->indices) + vertex_id);
}
__device__ __forceinline__ f3 load_position(uint64_t positions, uint32_t flags, uint32_t index) {
    if (flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>(positions) + (size_t)index * 3;
        return {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
    }
    const uint16_t* p = reinterpret_cast<const uint16_t*>(positions) + (size_t)index * 3;
    return {(float)__ldg(p), (float)__ldg(p + 1), (float)__ldg(p + 2)};
}
__device__ __forceinline__ f3 load_normal_raw(uint64_t normals, uint32_t flags, uint32_t index) {
    if (flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>(normals) + (size_t)index * 3;
        return {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
    }
    const int8_t* p = reinterpret_cast<const int8_t*>(normals) + (size_t)index * 3;
    return {(float)p[0], (float)p[1], (float)p[2]};
}
__device__ __forceinline__ f2 load_uv_raw(uint64_t uvs, uint32_t flags, uint32_t index) {
    if (flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>(uvs) + (size_t)index * 2;
        return {__ldg(p), __ldg(p + 1)};
    }
    const uint16_t* p = reinterpret_cast<const uint16_t*>(uvs) + (size_t)index * 2;
    return {(float)__ldg(p), (float)__ldg(p + 1)};
}
// Whole records with vector loads: Instance (112 B, 16-byte aligned array)
// and Meshlet (56 B, 8-byte aligned).
union InstanceBits {
    Instance inst;
    float4 v[7];
};
union MeshletBits {
    Meshlet m;
    uint2 v[7];
};
__device__ __forceinline__ void load_instance(const Instance* p, InstanceBits& out) {
    const float4* s = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < 7; i++) out.v[i] = __ldg(s + i);
}
__device__ __forceinline__ void load_meshlet(const Meshlet* p, MeshletBits& out) {
    const uint2* s = reinterpret_cast<const uint2*>(p);
#pragma unroll
    for (int i = 0; i < 7; i++) out.v[i] = __ldg(s + i);
}

__device__ __forceinline__ f3 world_pos(const lh_mat4& transform, f3 p) {
    f4 w = mul(transform, f4{p.x, p.y, p.z, 1.0f});
    return {w.x, w.y, w.z};
}

// Fields of a MeshInfo the resolve needs (loaded as aligned words).
struct MeshInfoResolve {
    uint64_t positions, indices, normals, uvs, micro_indices, meshlets;
    uint32_t flags;
    lh_vec2 texture_scale, texture_offset;
    uint32_t base_tex, mr_tex, normal_tex;
    lh_vec3 base_color_factor;
};
__device__ __forceinline__ MeshInfoResolve load_mesh_info_resolve(const MeshInfo* mi) {
    const unsigned long long* w = reinterpret_cast<const unsigned long long*>(mi);
    const uint32_t* d = reinterpret_cast<const uint32_t*>(mi);
    MeshInfoResolve r;
    r.positions = __ldg(w + 0);
    r.indices = __ldg(w + 1);
    r.normals = __ldg(w + 2);
    r.uvs = __ldg(w + 3);
    r.micro_indices = __ldg(w + 4);
    r.meshlets = __ldg(w + 5);
    r.flags = (uint32_t)((__ldg(w + 6) >> 16) & 0xFFu);
    r.texture_scale = {__uint_as_float(__ldg(d + 17)), __uint_as_float(__ldg(d + 18))};
    r.texture_offset = {__uint_as_float(__ldg(d + 19)), __uint_as_float(__ldg(d + 20))};
    uint32_t t01 = __ldg(d + 21), t2 = __ldg(d + 22);
    r.base_tex = t01 & 0xFFFFu;
    r.mr_tex = t01 >> 16;
    r.normal_tex = t2 & 0xFFFFu;
    r.base_color_factor = {__uint_as_float(__ldg(d + 23)), __uint_as_float(__ldg(d + 24)), __uint_as_float(__ldg(d + 25))};
    return r;
}


// ------------------------------------------------------------------ culling (culling.glsl)
__device__ __forceinline__ float max_scale(const lh_mat4& t) {
    float sx = length(f3{t.cols[0].x, t.cols[0].y, t.cols[0].z});
    float sy = length(f3{t.cols[1].x, t.cols[1].y, t.cols[1].z});
    float sz = length(f3{t.cols[2].x, t.cols[2].y, t.cols[2].z});
    return gmax(gmax(sx, sy), sz);
}

// culling.glsl:1-46; true = culled.
__device__ __forceinline__ bool cull_bounding_sphere(const Uniforms& u, const lh_mat4& transform, lh_vec4 bs) {
    f4 w4 = mul(transform, f4{bs.x, bs.y, bs.z, 1.0f});
    float radius = bs.w * max_scale(transform);
    f4 vs = mul(u.initial_view, f4{w4.x, w4.y, w4.z, 1.0f});
    vs.z = -vs.z;
    bool visible = vs.z + radius > NEAR_PLANE;
    const lh_mat4& P = u.perspective;
    f3 fx = normalize(f3{P.cols[0].w + P.cols[0].x, P.cols[1].w + P.cols[1].x, P.cols[2].w + P.cols[2].x});
    f3 fy = normalize(f3{P.cols[0].w + P.cols[0].y, P.cols[1].w + P.cols[1].y, P.cols[2].w + P.cols[2].y});
    visible = visible && vs.z * fx.z + fabsf(vs.x) * fx.x < radius;
    visible = visible && vs.z * fy.z - fabsf(vs.y) * fy.y < radius;
    return !visible;
}

// culling.glsl:48-135; true = culled.
__device__ __forceinline__ bool cull_bounding_sphere_shadows(const MiscStorage& m, const lh_mat4& transform,
                                                             lh_vec4 bs, uint32_t c) {
    f4 w4 = mul(transform, f4{bs.x, bs.y, bs.z, 1.0f});
    float radius = bs.w * max_scale(transform);
    f4 world{w4.x, w4.y, w4.z, 1.0f};
    f4 v = mul(m.shadow_view_matrices[c], world);
    float R = m.shadow_sphere_radii[c];
    if (!((fabsf(v.x) - radius < R) && (fabsf(v.y) - radius < R))) return true;
    for (uint32_t k = 0; k < c; k++) {
        f4 vk = mul(m.shadow_view_matrices[k], world);
        float Rk = m.shadow_sphere_radii[k];
        if ((fabsf(vk.x) + radius < Rk) && (fabsf(vk.y) + radius < Rk)) return true;
    }
    return false;
}

// culling.glsl:137-145
__device__ __forceinline__ bool cull_cone_perspective(const Uniforms& u, const Instance* inst, const lh_mat4& transform,
                                                      const Meshlet& ml) {
    f4 a4 = mul(transform, f4{ml.cone_apex.x, ml.cone_apex.y, ml.cone_apex.z, 1.0f});
    f3 axis = normalize(mul3(inst->normal_transform, ld3(ml.cone_axis)));
    return dot(normalize(f3{a4.x, a4.y, a4.z} - ld3(u.camera_pos)), normalize(axis)) >= ml.cone_cutoff;
}
// culling.glsl:147-151
__device__ __forceinline__ bool cull_cone_orthographic(const Uniforms& u, const Instance* inst, const Meshlet& ml) {
    f3 axis = normalize(mul3(inst->normal_transform, ld3(ml.cone_axis)));
    return dot(ld3(u.sun_dir), axis) >= ml.cone_cutoff;
}

// ------------------------------------------------------------------ rasterisation rules
// Outcode bits: 1 z > w (or w <= 0), 2 z < 0, 4 x > g*w, 8 x < -g*w,
// 16 y > g*w, 32 y < -g*w; 64 = a non-finite coordinate (the triangle is
// dropped).  Any other bit has the triangle clipped (clip_triangle).
__device__ __forceinline__ uint32_t outcode(f4 v) {
    if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w))) return 64u;
    uint32_t c = 0;
    float g = LH_GUARD_BAND * v.w;
    if (v.z > v.w || !(v.w > 0.0f)) c |= 1u;
    if (v.z < 0.0f) c |= 2u;
    if (v.x > g) c |= 4u;
    if (v.x < -g) c |= 8u;
    if (v.y > g) c |= 16u;
    if (v.y < -g) c |= 32u;
    return c;
}

struct SnapV { int32_t X, Y; float z; };

// Viewport transform + snap to 1/256 pixel (round to nearest even).  An
// orthographic view (the shadow cascades) has w = 1 exactly, and x / 1 = x
// for every x: the divides only run when they can change a bit.
__device__ __forceinline__ SnapV snap(f4 v, float hw, float hh) {
    float ndx = v.x, ndy = v.y;
    SnapV s;
    s.z = v.z;
    if (v.w != 1.0f) {
        ndx = v.x / v.w;
        ndy = v.y / v.w;
        s.z = v.z / v.w;
    }
    float xf = ndx * hw + hw, yf = ndy * hh + hh;
    s.X = __float2int_rn(xf * 256.0f);
    s.Y = __float2int_rn(yf * 256.0f);
    return s;
}

__device__ __forceinline__ int64_t cross3(const SnapV& a, const SnapV& b, const SnapV& c) {
    return ((int64_t)a.X * b.Y - (int64_t)b.X * a.Y) + ((int64_t)b.X * c.Y - (int64_t)c.X * b.Y) +
           ((int64_t)c.X * a.Y - (int64_t)a.X * c.Y);
}

// Twice the signed area (= cross3) from vertex differences: 32-bit products
// when every difference is below 2^15 in magnitude.
__device__ __forceinline__ int64_t cross_rel(const SnapV& a, const SnapV& b, const SnapV& c) {
    const int32_t ux = b.X - a.X, uy = b.Y - a.Y, vx = c.X - a.X, vy = c.Y - a.Y;
    if ((uint32_t)(ux + 0x7FFF) < 0xFFFFu && (uint32_t)(uy + 0x7FFF) < 0xFFFFu && (uint32_t)(vx + 0x7FFF) < 0xFFFFu &&
        (uint32_t)(vy + 0x7FFF) < 0xFFFFu)
        return (int64_t)(ux * vy - vx * uy);
    return (int64_t)ux * vy - (int64_t)vx * uy;
}

// Triangle ready for coverage: orientation normalised (interior has every
// edge function >= 0), bias 1 for edges that are not top-left.
struct TriSetup {
    int32_t X0, Y0, X1, Y1, X2, Y2;
    float z0, s1, s2;
    uint32_t id;
    int32_t px0, py0, px1, py1;
    uint32_t bias;  // bit0 edge12, bit1 edge20, bit2 edge01 not top-left;
                    // bit3: every edge product in the bbox fits 32 bits;
                    // bit4 (kBiasAlpha): alpha-tested
    uint32_t verts;  // alpha-tested: meshlet vertices m0 | m1 << 8 | m2 << 16
};
constexpr uint32_t kBiasAlpha = 16u;

__device__ __forceinline__ bool top_left(int32_t ax, int32_t ay, int32_t bx, int32_t by) {
    int32_t dy = by - ay, dx = bx - ax;
    return dy > 0 || (dy == 0 && dx < 0);
}

// Pixel bbox of a triangle in a W x H target (the pixel centres its snapped
// vertex extents can hold) and the extents themselves.
struct TriBox {
    int32_t px0, px1, py0, py1;
    int32_t ext_x, ext_y;  // snapped vertex extents (1/256 pixel)
};
__device__ __forceinline__ TriBox tri_box(const SnapV& v0, const SnapV& v1, const SnapV& v2, uint32_t W, uint32_t H) {
    const int32_t minX = min(v0.X, min(v1.X, v2.X)), maxX = max(v0.X, max(v1.X, v2.X));
    const int32_t minY = min(v0.Y, min(v1.Y, v2.Y)), maxY = max(v0.Y, max(v1.Y, v2.Y));
    TriBox b;
    b.px0 = max((minX + 127) >> 8, 0);
    b.px1 = min((maxX - 128) >> 8, (int32_t)W - 1);
    b.py0 = max((minY + 127) >> 8, 0);
    b.py1 = min((maxY - 128) >> 8, (int32_t)H - 1);
    b.ext_x = maxX - minX;
    b.ext_y = maxY - minY;
    return b;
}
__device__ __forceinline__ bool box_empty(const TriBox& b) { return b.px0 > b.px1 || b.py0 > b.py1; }

// The rest of the setup once the orientation is normalised and the doubled
// area A > 0 and the (non-empty) box are known.
__device__ __forceinline__ void finish_setup(SnapV v0, SnapV v1, SnapV v2, int64_t A, const TriBox& b, uint32_t id,
                                             TriSetup& t) {
    t.px0 = b.px0;
    t.px1 = b.px1;
    t.py0 = b.py0;
    t.py1 = b.py1;
    t.X0 = v0.X; t.Y0 = v0.Y; t.X1 = v1.X; t.Y1 = v1.Y; t.X2 = v2.X; t.Y2 = v2.Y;
    // A > 0 (round to nearest even either way; FP32 adds below 2^46)
    const float fA = A < (1ll << 46) ? u46_to_f32_rn((uint64_t)A) : __ll2float_rn(A);
    t.z0 = v0.z;
    t.s1 = (v1.z - v0.z) / fA;
    t.s2 = (v2.z - v0.z) / fA;
    t.id = id;
    t.bias = (top_left(v1.X, v1.Y, v2.X, v2.Y) ? 0u : 1u) | (top_left(v2.X, v2.Y, v0.X, v0.Y) ? 0u : 2u) |
             (top_left(v0.X, v0.Y, v1.X, v1.Y) ? 0u : 4u);
    // pixel centres of the bbox lie inside the vertex extents, so each
    // product of an edge function is at most ext_x * ext_y in magnitude
    // (and, so that per-pixel steps of 256 units fit too, both extents are
    // below 2^22)
    if ((int64_t)b.ext_x * (int64_t)b.ext_y < (1ll << 30) && b.ext_x < (1 << 22) && b.ext_y < (1 << 22))
        t.bias |= 8u;
}

// Build the setup of a normalised triangle; returns false when no pixel
// centre of the (W x H) target can be covered.
__device__ __forceinline__ bool make_setup(SnapV v0, SnapV v1, SnapV v2, uint32_t id, uint32_t W, uint32_t H,
                                           TriSetup& t) {
    int64_t A = (int64_t)(v2.Y - v1.Y) * (v0.X - v1.X) - (int64_t)(v2.X - v1.X) * (v0.Y - v1.Y);
    if (A <= 0) return false;
    const TriBox b = tri_box(v0, v1, v2, W, H);
    if (box_empty(b)) return false;
    finish_setup(v0, v1, v2, A, b, id, t);
    return true;
}

// An edge function value as float (round to nearest even): the 32-bit route
// when it fits, else the conversion instruction (LH_EDGE_CONV=2: the
// integer-only routine; same bits either way).
#ifndef LH_EDGE_CONV
#define LH_EDGE_CONV 1
#endif
__device__ __forceinline__ float edge_to_float(int64_t e) {
    if (e == (int64_t)(int32_t)e) return i32_to_f32_rn((int32_t)e);
#if LH_EDGE_CONV == 2
    return i64_to_f32_rn(e);
#else
    return __ll2float_rn(e);
#endif
}

// The three edge functions of a small triangle (bias bit 3) at the centre
// of its bbox's first pixel and their steps per pixel in x and y: the
// function at pixel (px0 + rx, py0 + ry) is e0 + rx * dx + ry * dy, the same
// integer cover() forms, with every partial sum inside the 32-bit range.
struct EdgeSteps {
    int32_t e0[3], dx[3], dy[3];
};
__device__ __forceinline__ EdgeSteps edge_steps(const TriSetup& t) {
    const int32_t Px = t.px0 * 256 + 128, Py = t.py0 * 256 + 128;
    EdgeSteps s;
    s.e0[0] = (t.Y2 - t.Y1) * (Px - t.X1) - (t.X2 - t.X1) * (Py - t.Y1);
    s.e0[1] = (t.Y0 - t.Y2) * (Px - t.X2) - (t.X0 - t.X2) * (Py - t.Y2);
    s.e0[2] = (t.Y1 - t.Y0) * (Px - t.X0) - (t.X1 - t.X0) * (Py - t.Y0);
    s.dx[0] = (t.Y2 - t.Y1) * 256;
    s.dx[1] = (t.Y0 - t.Y2) * 256;
    s.dx[2] = (t.Y1 - t.Y0) * 256;
    s.dy[0] = -(t.X2 - t.X1) * 256;
    s.dy[1] = -(t.X0 - t.X2) * 256;
    s.dy[2] = -(t.X1 - t.X0) * 256;
    return s;
}
__device__ __forceinline__ bool cover_step(const TriSetup& t, const EdgeSteps& s, int32_t rx, int32_t ry,
                                           float& depth) {
    const int32_t e12 = s.e0[0] + rx * s.dx[0] + ry * s.dy[0];
    const int32_t e20 = s.e0[1] + rx * s.dx[1] + ry * s.dy[1];
    const int32_t e01 = s.e0[2] + rx * s.dx[2] + ry * s.dy[2];
    if (e12 < (int32_t)(t.bias & 1u) || e20 < (int32_t)((t.bias >> 1) & 1u) || e01 < (int32_t)((t.bias >> 2) & 1u))
        return false;
    float d = (t.z0 + i32_to_f32_rn(e20) * t.s1) + i32_to_f32_rn(e01) * t.s2;
    d = d > 0.0f ? d : 0.0f;
    depth = d < 1.0f ? d : 1.0f;
    return true;
}

// Coverage + depth of pixel (px, py); returns false when not covered.
__device__ __forceinline__ bool cover(const TriSetup& t, int32_t px, int32_t py, float& depth) {
    float f20, f01;
    if (t.bias & 8u) {
        const int32_t Px = px * 256 + 128, Py = py * 256 + 128;
        const int32_t e12 = (t.Y2 - t.Y1) * (Px - t.X1) - (t.X2 - t.X1) * (Py - t.Y1);
        const int32_t e20 = (t.Y0 - t.Y2) * (Px - t.X2) - (t.X0 - t.X2) * (Py - t.Y2);
        const int32_t e01 = (t.Y1 - t.Y0) * (Px - t.X0) - (t.X1 - t.X0) * (Py - t.Y0);
        if (e12 < (int32_t)(t.bias & 1u) || e20 < (int32_t)((t.bias >> 1) & 1u) ||
            e01 < (int32_t)((t.bias >> 2) & 1u))
            return false;
        f20 = i32_to_f32_rn(e20);
        f01 = i32_to_f32_rn(e01);
    } else {
        const int64_t Px = (int64_t)px * 256 + 128, Py = (int64_t)py * 256 + 128;
        const int64_t e12 = (int64_t)(t.Y2 - t.Y1) * (Px - t.X1) - (int64_t)(t.X2 - t.X1) * (Py - t.Y1);
        const int64_t e20 = (int64_t)(t.Y0 - t.Y2) * (Px - t.X2) - (int64_t)(t.X0 - t.X2) * (Py - t.Y2);
        const int64_t e01 = (int64_t)(t.Y1 - t.Y0) * (Px - t.X0) - (int64_t)(t.X1 - t.X0) * (Py - t.Y0);
        if (e12 < (int64_t)(t.bias & 1u) || e20 < (int64_t)((t.bias >> 1) & 1u) ||
            e01 < (int64_t)((t.bias >> 2) & 1u))
            return false;
        f20 = edge_to_float(e20);
        f01 = edge_to_float(e01);
    }
    float d = (t.z0 + f20 * t.s1) + f01 * t.s2;
    d = d > 0.0f ? d : 0.0f;
    depth = d < 1.0f ? d : 1.0f;
    return true;
}

// Depth test + write: kind 0 keeps the max of (depth bits << 32 | id) in a
// u64 visibility target (reverse-Z GREATER), kind 1 keeps the min of depth
// bits in a u32 shadow target (LESS).  The atomics return nothing (RED), so
// a warp never waits on the L2 round trip of a fragment.
template <int KIND>
__device__ __forceinline__ void write_fragment(void* target, uint32_t W, int32_t px, int32_t py, float depth,
                                               uint32_t id) {
    size_t pix = (size_t)py * W + px;
    if (KIND == 0) {
        const unsigned long long key = ((unsigned long long)f2u(depth) << 32) | id;
        asm volatile("red.relaxed.gpu.global.max.u64 [%0], %1;" ::"l"(reinterpret_cast<unsigned long long*>(target) + pix),
                     "l"(key));
    } else {
        asm volatile("red.relaxed.gpu.global.min.u32 [%0], %1;" ::"l"(reinterpret_cast<uint32_t*>(target) + pix),
                     "r"(f2u(depth)));
    }
}

// One pixel of the HDR target: RGBA32F, or RGBA16F (round to nearest even,
// the reference's format) when the context asks for it.  Streaming stores:
// nothing re-reads the image in the frame.
__device__ __forceinline__ void store_hdr(void* hdr, uint32_t half, size_t pixel, float r, float g, float b) {
    if (half) {
        const __half2 rg = __floats2half2_rn(r, g), ba = __floats2half2_rn(b, 1.0f);
        uint2 v;
        v.x = *reinterpret_cast<const uint32_t*>(&rg);
        v.y = *reinterpret_cast<const uint32_t*>(&ba);
        __stcs(reinterpret_cast<uint2*>(hdr) + pixel, v);
    } else {
        __stcs(reinterpret_cast<float4*>(hdr) + pixel, make_float4(r, g, b, 1.0f));
    }
}
__device__ __forceinline__ float4 load_hdr(const void* hdr, uint32_t half, size_t pixel) {
    if (half) {
        const uint2 v = __ldcs(reinterpret_cast<const uint2*>(hdr) + pixel);
        const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
        const float2 ba = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
        return make_float4(rg.x, rg.y, ba.x, ba.y);
    }
    return __ldcs(reinterpret_cast<const float4*>(hdr) + pixel);
}

}  // namespace lh
