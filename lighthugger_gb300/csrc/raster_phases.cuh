// Compute rasteriser for the visibility buffer and the cascade shadow maps.
//
// Replaces the reference's hardware draws: visbuffer_opaque_vertex/pixel
// (src/shaders/rasterization.glsl:12-58) with depth GREATER / clear 0 /
// back-face culling (src/pipelines.cpp:10-13,67-71,287-300), and
// shadowmap_opaque_vertex (rasterization.glsl:101-111) with depth LESS /
// clear 1 / front-face culling (pipelines.cpp:15-19,73-77,257-270), driven
// by drawIndirectCount over the draw lists (src/rendering.cpp:197-266,
// 325-438).  Alpha-clip draws (visbuffer_alpha_clip_vertex/pixel and
// shadowmap_alpha_clip*, rasterization.glsl:60-97,113-145) are double sided
// (pipelines.cpp:272-285,302-315) and alpha tested per fragment: the base
// texture's alpha, sampled bilinearly at the perspective-correct uv of the
// pixel centre, must not be below 0.5.
//
// Layout of the work:
//  k_raster       one warp per visible meshlet (claimed dynamically across
//                 all views of the launch): the meshlet's <= 64 vertices are
//                 transformed once, snapped to 1/256 px and kept in shared
//                 memory; then one lane per triangle does set-up and face
//                 culling.  Triangles covering <= `small` pixel centres are
//                 rasterised by their lane, up to `medium` by the whole warp,
//                 larger ones go to a queue of chunks (tiles of the bbox).
//                 A triangle that needs clipping is clipped by its lane
//                 (Sutherland-Hodgman in clip space against 0 <= z <= w and
//                 the guard band, fan triangulation) into the chunk queue.
//  k_raster_big   one warp per chunk: each row's run of covered pixels
//                 from the three edge functions, the runs walked row by
//                 row or compacted across the warp.
// The depth test is an atomicMax of (depth bits << 32 | packed ID) for the
// visibility buffer and an atomicMin of depth bits for shadow maps, so the
// result does not depend on the order of the work.
#pragma once

#include <type_traits>

#include "edge_run.cuh"
#include "lh_device.cuh"
#include "lh_internal.cuh"

namespace lh {
namespace {

constexpr int kRasterWarps = 8;

// Chunks of big triangles a warp claims per atomic (build knob; large
// frame 0.395 ms at 2, 0.397 at 4, 0.425 at 1, 0.464 at 8).
#ifndef LH_CHUNK_BATCH
#define LH_CHUNK_BATCH 2
#endif

// Upper bound of the warp bin in the shadow pass (0: the tuning's medium_px
// for both passes).  A shadow launch has about one unit per warp, so a warp
// that rasterises a run of 33-128-pixel triangles one after another sets the
// launch's time; sent to the chunk kernel instead, they spread over all
// warps: shadow raster stage 0.099 -> 0.087 ms at 32 (0.096 ms at 64) for the
// four 1024^2 cascades of the 4,096-instance frame.
#ifndef LH_SHADOW_MEDIUM_PX
#define LH_SHADOW_MEDIUM_PX 32
#endif

struct RasterTune {
    uint32_t small_px;   // lane path up to this many bbox pixels
    uint32_t medium_px;  // warp path up to this many; larger: chunk queue
    uint32_t batch;      // meshlets claimed per atomic (0: automatic)
};

__device__ __forceinline__ const lh_mat4& view_matrix(const FrameDev& f, const ViewDev* vw) {
    return vw->kind == kViewVisibility ? vw->uniforms->combined_perspective_view : f.misc->shadow_matrices[vw->cascade];
}

// Fields of a MeshInfo the raster needs.
struct MeshInfoRaster {
    uint64_t positions, indices, micro_indices, meshlets;
    uint32_t flags;
};
__device__ __forceinline__ MeshInfoRaster load_mesh_info_raster(const MeshInfo* mi) {
    const unsigned long long* w = reinterpret_cast<const unsigned long long*>(mi);
    MeshInfoRaster r;
    r.positions = __ldg(w + 0);
    r.indices = __ldg(w + 1);
    r.micro_indices = __ldg(w + 4);
    r.meshlets = __ldg(w + 5);
    r.flags = (uint32_t)((__ldg(w + 6) >> 16) & 0xFFu);
    return r;
}

// ------------------------------------------------------------ alpha clip
// One vertex of an alpha-tested triangle: clip x, y, w and the uv the
// reference's vertex shader forms (uv * texture_scale + texture_offset).
struct AlphaVert {
    float x, y, w, u, v;
};

// Fields of a MeshInfo the alpha test needs.
struct MeshInfoAlpha {
    uint64_t uvs;
    float ts_x, ts_y, to_x, to_y;
    uint32_t tex;
};
__device__ __forceinline__ MeshInfoAlpha load_mesh_info_alpha(const MeshInfo* mi) {
    MeshInfoAlpha r;
    r.uvs = __ldg(&mi->uvs);
    r.ts_x = __ldg(&mi->texture_scale.x);
    r.ts_y = __ldg(&mi->texture_scale.y);
    r.to_x = __ldg(&mi->texture_offset.x);
    r.to_y = __ldg(&mi->texture_offset.y);
    r.tex = __ldg(&mi->base_color_texture_index);
    return r;
}
__device__ __forceinline__ AlphaVert alpha_vert(f4 c, const MeshInfoAlpha& ma, uint32_t flags, uint32_t index) {
    const f2 uv = load_uv_raw(ma.uvs, flags, index);
    return AlphaVert{c.x, c.y, c.w, uv.x * ma.ts_x + ma.to_x, uv.y * ma.ts_y + ma.to_y};
}

// 2D homogeneous edge functions of the unclipped triangle (Olano and Greer,
// "Triangle scan conversion using 2D homogeneous coordinates", 1997):
// E_k(nx, ny) = a_k nx + b_k ny + c_k with (a_k, b_k, c_k) = v_i x v_j for
// (i, j) = (1, 2), (2, 0), (0, 1) over v = (x, y, w); the perspective-correct
// barycentrics are E_k / (E_0 + E_1 + E_2), for clipped triangles too.
struct AlphaTri {
    float a[3], b[3], c[3];
    float u[3], v[3];
    uint32_t tex;
};
__device__ __forceinline__ void alpha_edge(const AlphaVert& p, const AlphaVert& q, float& a, float& b, float& c) {
    a = p.y * q.w - q.y * p.w;
    b = p.w * q.x - q.w * p.x;
    c = p.x * q.y - q.x * p.y;
}
__device__ __forceinline__ AlphaTri alpha_setup(const AlphaVert& v0, const AlphaVert& v1, const AlphaVert& v2,
                                                uint32_t tex) {
    AlphaTri t;
    alpha_edge(v1, v2, t.a[0], t.b[0], t.c[0]);
    alpha_edge(v2, v0, t.a[1], t.b[1], t.c[1]);
    alpha_edge(v0, v1, t.a[2], t.b[2], t.c[2]);
    t.u[0] = v0.u;
    t.u[1] = v1.u;
    t.u[2] = v2.u;
    t.v[0] = v0.v;
    t.v[1] = v1.v;
    t.v[2] = v2.v;
    t.tex = tex;
    return t;
}

// Alpha of the bilinear, repeat-addressed sample of texture `index` at uv.
__device__ __forceinline__ float sample_alpha(const FrameDev& f, uint32_t index, float uvx, float uvy) {
    if (index >= f.n_textures) return 0.0f;
    const lh_texture t = f.textures[index];
    const float4* tex = f.tex_linear[index];
    float u = uvx * (float)t.width - 0.5f, v = uvy * (float)t.height - 0.5f;
    if (!(fabsf(u) < 1e9f)) u = 0.0f;
    if (!(fabsf(v) < 1e9f)) v = 0.0f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int32_t i0 = (int32_t)fu, j0 = (int32_t)fv, W = (int32_t)t.width, H = (int32_t)t.height;
    const int32_t ia = wrap_texel(i0, W), ib = wrap_texel(i0 + 1, W), ja = wrap_texel(j0, H), jb = wrap_texel(j0 + 1, H);
    auto al = [&](int32_t i, int32_t j) { return __ldg(&tex[(size_t)j * W + i].w); };
    const float t00 = al(ia, ja), t10 = al(ib, ja), t01 = al(ia, jb), t11 = al(ib, jb);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return ((t00 * w00 + t10 * w10) + t01 * w01) + t11 * w11;
}

// True when the fragment at pixel (px, py) of a W x H target survives.
__device__ __forceinline__ bool alpha_pass(const FrameDev& f, const AlphaTri& t, int32_t px, int32_t py, uint32_t W,
                                           uint32_t H) {
    const float nx = (((float)px + 0.5f) / (float)W) * 2.0f - 1.0f;
    const float ny = (((float)py + 0.5f) / (float)H) * 2.0f - 1.0f;
    const float e0 = (t.a[0] * nx + t.b[0] * ny) + t.c[0];
    const float e1 = (t.a[1] * nx + t.b[1] * ny) + t.c[1];
    const float e2 = (t.a[2] * nx + t.b[2] * ny) + t.c[2];
    const float sum = (e0 + e1) + e2;
    const float l0 = e0 / sum, l1 = e1 / sum, l2 = e2 / sum;
    const float u = (l0 * t.u[0] + l1 * t.u[1]) + l2 * t.u[2];
    const float v = (l0 * t.v[0] + l1 * t.v[1]) + l2 * t.v[2];
    return !(sample_alpha(f, t.tex, u, v) < 0.5f);
}

// The alpha set-up of triangle `id` (packed tri / draw slot) of view
// `view`, from the scene buffers (the chunk and clip paths).
__device__ AlphaTri alpha_tri_global(const FrameDev& f, uint32_t view, uint32_t id) {
    const ViewDev* vw = f.views + view;
    const uint32_t slot = id & ((1u << 24) - 1u), tri = id >> 24;
    const MeshletReference ref = vw->refs[slot];
    const Instance* inst = f.instances + ref.instance_index;
    lh_mat4 transform;
    const float4* src = reinterpret_cast<const float4*>(inst);
    float4* dst = reinterpret_cast<float4*>(&transform);
    for (int i = 0; i < 4; i++) dst[i] = __ldg(src + i);
    const MeshInfo* mip = mesh_info_of(inst);
    const MeshInfoRaster mi = load_mesh_info_raster(mip);
    const MeshInfoAlpha ma = load_mesh_info_alpha(mip);
    const Meshlet* ml = reinterpret_cast<const Meshlet*>(mi.meshlets) + ref.meshlet_index;
    const uint32_t tri_off = __ldg(&ml->triangle_offset), idx_off = __ldg(&ml->index_offset);
    const uint8_t* micro = reinterpret_cast<const uint8_t*>(mi.micro_indices) + tri_off + tri * 3;
    const lh_mat4& vp = view_matrix(f, vw);
    AlphaVert av[3];
    for (int k = 0; k < 3; k++) {
        const uint32_t idx = (mi.flags & MESH_INFO_FLAGS_32_BIT_INDICES)
                                 ? __ldg(reinterpret_cast<const uint32_t*>(mi.indices) + idx_off + __ldg(micro + k))
                                 : __ldg(reinterpret_cast<const uint16_t*>(mi.indices) + idx_off + __ldg(micro + k));
        const f3 w = world_pos(transform, load_position(mi.positions, mi.flags, idx));
        av[k] = alpha_vert(mul(vp, f4{w.x, w.y, w.z, 1.0f}), ma, mi.flags, idx);
    }
    return alpha_setup(av[0], av[1], av[2], ma.tex);
}
__device__ __forceinline__ uint32_t load_index_raw(uint64_t indices, uint32_t flags, uint32_t i) {
    if (flags & MESH_INFO_FLAGS_32_BIT_INDICES) return __ldg(reinterpret_cast<const uint32_t*>(indices) + i);
    return __ldg(reinterpret_cast<const uint16_t*>(indices) + i);
}

__device__ __forceinline__ void load_transform(const Instance* inst, lh_mat4& m) {
    const float4* s = reinterpret_cast<const float4*>(inst);
    float4* d = reinterpret_cast<float4*>(&m);
#pragma unroll
    for (int i = 0; i < 4; i++) d[i] = __ldg(s + i);
}

// Append big triangles with 64-bit atomics of {triangles:hi24, chunks:lo40}
// (the packed single-pass append of prefix_sum.glsl:17-30): the triangle's
// index and its first chunk come from the same word, so chunk bases ascend
// with the index and the chunk kernel finds a chunk's triangle by binary search.
template <int KIND>
__device__ __forceinline__ unsigned long long big_chunks(const FrameDev& f, const TriSetup& t) {
    const uint32_t nbx = ((uint32_t)(t.px1 - t.px0) >> f.chunk_shift[KIND][1]) + 1;
    const uint32_t nby = ((uint32_t)(t.py1 - t.py0) >> f.chunk_shift[KIND][0]) + 1;
    return (unsigned long long)nbx * nby;
}
// Store the queue entry of a triangle of n chunks whose packed word (before
// its own addition) is `old`.
__device__ void store_big(const FrameDev& f, const TriSetup& t, uint32_t view, unsigned long long old,
                          unsigned long long n) {
    const uint64_t idx = old >> 40, base = old & ((1ull << 40) - 1);
    if (idx >= f.big_cap || base + n > 0xFFFFFFFFull) {
        atomicOr(&f.status[kStFlags], LH_FLAG_QUEUE_OVERFLOW);
        return;
    }
    BigTri e;
    e.X0 = t.X0; e.Y0 = t.Y0; e.X1 = t.X1; e.Y1 = t.Y1; e.X2 = t.X2; e.Y2 = t.Y2;
    e.z0 = t.z0; e.s1 = t.s1; e.s2 = t.s2;
    e.id = t.id;
    e.view = view;
    e.bias = t.bias;
    e.px0 = t.px0;
    e.px1 = t.px1;
    e.py0 = t.py0;
    e.py1 = t.py1;
    f.big[idx] = e;
    f.big_base[idx] = (uint32_t)base;
}
// One thread's triangle.
template <int KIND>
__device__ void push_big(const FrameDev& f, const TriSetup& t, uint32_t view) {
    const unsigned long long n = big_chunks<KIND>(f, t);
    const unsigned long long old =
        atomicAdd(reinterpret_cast<unsigned long long*>(f.status + kStBigPacked), (1ull << 40) | n);
    store_big(f, t, view, old, n);
}
// Called by the whole warp: lanes with `big` set append their triangle with
// one atomic per warp (a warp scan of the lanes' {1, chunks} words gives each
// lane the running total below it).  The word's low 40 bits cannot carry into
// the count: a sum reaching 2^32 chunks is flagged and dropped.
template <int KIND>
__device__ void push_big_warp(const FrameDev& f, const TriSetup& t, uint32_t view, bool big, uint32_t lane) {
    const unsigned long long n = big ? big_chunks<KIND>(f, t) : 0ull;
    const unsigned long long mine = big ? (1ull << 40) | n : 0ull;
    unsigned long long incl = mine;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    unsigned long long old = 0;
    if (lane == 31) old = atomicAdd(reinterpret_cast<unsigned long long*>(f.status + kStBigPacked), incl);
    old = __shfl_sync(0xFFFFFFFFu, old, 31) + (incl - mine);
    if (big) store_big(f, t, view, old, n);
}

// Sutherland-Hodgman against w-z, z, g*w-x, g*w+x, g*w-y, g*w+y >= 0.
__device__ int clip_polygon(f4* poly, int n) {
    f4 out[9];
    for (int plane = 0; plane < 6 && n >= 3; plane++) {
        int m = 0;
        for (int i = 0; i < n; i++) {
            f4 a = poly[i], b = poly[i + 1 < n ? i + 1 : 0];
            float ga = LH_GUARD_BAND * a.w, gb = LH_GUARD_BAND * b.w;
            float da, db;
            switch (plane) {
                case 0: da = a.w - a.z; db = b.w - b.z; break;
                case 1: da = a.z; db = b.z; break;
                case 2: da = ga - a.x; db = gb - b.x; break;
                case 3: da = ga + a.x; db = gb + b.x; break;
                case 4: da = ga - a.y; db = gb - b.y; break;
                default: da = ga + a.y; db = gb + b.y; break;
            }
            if (da >= 0.0f) out[m++] = a;
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float tt = da / (da - db);
                out[m++] = f4{a.x + tt * (b.x - a.x), a.y + tt * (b.y - a.y), a.z + tt * (b.z - a.z), a.w + tt * (b.w - a.w)};
            }
        }
        n = m;
        for (int i = 0; i < n; i++) poly[i] = out[i];
    }
    return n;
}

// Triangle `tri` of the meshlet at draw slot `slot` of view `view`, one of
// whose vertices lies outside 0 <= z <= w, w > 0 or the guard band: clipped
// in clip space, fan-triangulated, the pieces appended to the chunk queue.
// Called by the lane that found it during the raster (rare, so the
// polygon's stack arrays stay out of the raster's register allocation).
template <int KIND>
__device__ __noinline__ void clip_triangle(const FrameDev& f, uint32_t view, uint32_t slot, uint32_t tri) {
    {
        const struct { uint32_t view, slot, tri; } it{view, slot, tri};
        const ViewDev* vw = f.views + it.view;
        const MeshletReference ref = vw->refs[it.slot];
        const Instance* inst = f.instances + ref.instance_index;
        lh_mat4 transform;
        load_transform(inst, transform);
        const MeshInfoRaster mi = load_mesh_info_raster(mesh_info_of(inst));
        MeshletBits mb;
        load_meshlet(reinterpret_cast<const Meshlet*>(mi.meshlets) + ref.meshlet_index, mb);
        const lh_mat4& vp = view_matrix(f, vw);
        const uint8_t* micro = reinterpret_cast<const uint8_t*>(mi.micro_indices) + mb.m.triangle_offset + it.tri * 3;
        const bool alpha = it.slot >= f.max_draws;  // alpha clip: double sided, alpha tested
        f4 poly[9];
        for (int k = 0; k < 3; k++) {
            uint32_t idx = load_index_raw(mi.indices, mi.flags, mb.m.index_offset + micro[k]);
            f3 w = world_pos(transform, load_position(mi.positions, mi.flags, idx));
            poly[k] = mul(vp, f4{w.x, w.y, w.z, 1.0f});
        }
        int np = clip_polygon(poly, 3);
        if (np < 3) return;
        bool projectable = true;  // false only for a triangle through the eye point
        for (int k = 0; k < np; k++) projectable = projectable && poly[k].w > 0.0f;
        if (!projectable) return;
        const uint32_t W = vw->width, H = vw->height;
        const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
        SnapV s[9];
        for (int k = 0; k < np; k++) s[k] = snap(poly[k], hw, hh);
        int64_t pc = 0;
        for (int k = 0; k < np; k++) {
            const SnapV &a = s[k], &b = s[k + 1 < np ? k + 1 : 0];
            pc += (int64_t)a.X * b.Y - (int64_t)b.X * a.Y;
        }
        if (pc == 0) return;
        if (!alpha && KIND == 0 && pc > 0) return;
        if (!alpha && KIND == 1 && pc < 0) return;
        const uint32_t id = LH_PACK_ID(it.tri, it.slot);
        for (int k = 1; k + 1 < np; k++) {
            SnapV a = s[0], b = s[k], c = s[k + 1];
            int64_t tc = cross3(a, b, c);
            if (tc == 0 || ((tc < 0) != (pc < 0))) continue;
            if (tc > 0) { SnapV tmp = b; b = c; c = tmp; }
            TriSetup st;
            if (make_setup(a, b, c, id, W, H, st)) {
                if (alpha) st.bias |= kBiasAlpha;
                push_big<KIND>(f, st, it.view);
            }
        }
    }
}

// Where a warp's alpha-tested triangles find their vertices: the warp's
// shared AlphaVert array (indexed by TriSetup::verts) and the meshlet's
// base texture.
struct AlphaSrc {
    const AlphaVert* av;
    uint32_t tex;
    uint32_t H;
};

__device__ __forceinline__ AlphaTri alpha_of(const TriSetup& t, const AlphaSrc& as) {
    return alpha_setup(as.av[t.verts & 0xFFu], as.av[(t.verts >> 8) & 0xFFu], as.av[(t.verts >> 16) & 0xFFu], as.tex);
}

// The bbox pixels of one triangle by one lane; `nfrag` counts the fragments
// written (depth-test reductions issued).
template <int KIND>
__device__ __forceinline__ void raster_lane(const TriSetup& t, void* target, uint32_t W, uint32_t& nfrag) {
    if (t.bias & 8u) {
        const EdgeSteps es = edge_steps(t);
        for (int32_t ry = 0; ry <= t.py1 - t.py0; ry++)
            for (int32_t rx = 0; rx <= t.px1 - t.px0; rx++) {
                float d;
                if (cover_step(t, es, rx, ry, d)) {
                    write_fragment<KIND>(target, W, t.px0 + rx, t.py0 + ry, d, t.id);
                    nfrag++;
                }
            }
        return;
    }
    for (int32_t py = t.py0; py <= t.py1; py++)
        for (int32_t px = t.px0; px <= t.px1; px++) {
            float d;
            if (cover(t, px, py, d)) {
                write_fragment<KIND>(target, W, px, py, d, t.id);
                nfrag++;
            }
        }
}

// All lanes of a warp cover the pixels of one triangle's bbox.
template <int KIND>
__device__ __forceinline__ void raster_warp(const TriSetup& t, void* target, uint32_t W, uint32_t lane,
                                            uint32_t& nfrag) {
    const uint32_t w = (uint32_t)(t.px1 - t.px0 + 1);
    const uint32_t npx = w * (uint32_t)(t.py1 - t.py0 + 1);
    const float inv_w = 1.0f / (float)w;
    for (uint32_t p = lane; p < npx; p += 32) {
        int32_t ry = (int32_t)(((float)p + 0.5f) * inv_w);
        int32_t rx = (int32_t)p - ry * (int32_t)w;
        if (rx < 0) { ry--; rx += (int32_t)w; }
        else if (rx >= (int32_t)w) { ry++; rx -= (int32_t)w; }
        int32_t px = t.px0 + rx, py = t.py0 + ry;
        float d;
        if (cover(t, px, py, d)) {
            write_fragment<KIND>(target, W, px, py, d, t.id);
            nfrag++;
        }
    }
}

// The alpha-tested variants are not inlined: their set-up and sampling
// state stays out of the register allocation of the opaque paths (the
// launch bounds cap the whole call tree; alpha triangles are the rare case).
template <int KIND>
__device__ __noinline__ uint32_t raster_lane_alpha(const FrameDev& f, const TriSetup& t, void* target, uint32_t W,
                                                   const AlphaSrc& as) {
    const AlphaTri at = alpha_of(t, as);
    uint32_t n = 0;
    for (int32_t py = t.py0; py <= t.py1; py++)
        for (int32_t px = t.px0; px <= t.px1; px++) {
            float d;
            if (cover(t, px, py, d) && alpha_pass(f, at, px, py, W, as.H)) {
                write_fragment<KIND>(target, W, px, py, d, t.id);
                n++;
            }
        }
    return n;
}

template <int KIND>
__device__ __noinline__ uint32_t raster_warp_alpha(const FrameDev& f, const TriSetup& t, void* target, uint32_t W,
                                                   uint32_t lane, const AlphaSrc& as) {
    const uint32_t w = (uint32_t)(t.px1 - t.px0 + 1);
    const uint32_t npx = w * (uint32_t)(t.py1 - t.py0 + 1);
    const float inv_w = 1.0f / (float)w;
    const AlphaTri at = alpha_of(t, as);
    uint32_t n = 0;
    for (uint32_t p = lane; p < npx; p += 32) {
        int32_t ry = (int32_t)(((float)p + 0.5f) * inv_w);
        int32_t rx = (int32_t)p - ry * (int32_t)w;
        if (rx < 0) { ry--; rx += (int32_t)w; }
        else if (rx >= (int32_t)w) { ry++; rx -= (int32_t)w; }
        int32_t px = t.px0 + rx, py = t.py0 + ry;
        float d;
        if (cover(t, px, py, d) && alpha_pass(f, at, px, py, W, as.H)) {
            write_fragment<KIND>(target, W, px, py, d, t.id);
            n++;
        }
    }
    return n;
}

__device__ __forceinline__ TriSetup shfl_setup(const TriSetup& s, int src) {
    TriSetup r;
    const uint32_t* a = reinterpret_cast<const uint32_t*>(&s);
    uint32_t* b = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(TriSetup) / 4); i++) b[i] = __shfl_sync(0xFFFFFFFFu, a[i], src);
    return r;
}

// Shared memory of the raster phase (declared by the calling kernel, so that
// the persistent kernel's phases reuse one copy).  The alpha-clip class adds
// an AlphaVert array per warp (RasterSmemAlpha).
constexpr uint32_t kMicroWords = (MAX_MESHLET_TRIANGLES * 3 + 3) / 4;
struct RasterSmem {
    uint32_t prefix[kMaxViews + 1];
    __align__(16) lh_mat4 vp[kMaxViews];
    SnapV v[kRasterWarps][MAX_MESHLET_UNIQUE_VERTICES];
    uint8_t oc[kRasterWarps][MAX_MESHLET_UNIQUE_VERTICES];
    uint32_t micro[kRasterWarps][kMicroWords];
};
struct RasterSmemAlpha : RasterSmem {
    AlphaVert av[kRasterWarps][MAX_MESHLET_UNIQUE_VERTICES];
};

// One claimed meshlet (or quarter of one) of a view, as the warp works on it.
struct MeshletWork {
    uint32_t view, slot, part, split, nv, nt, W, H;
    void* target;
    float hw, hh;
    const lh_mat4* vp;  // the view's matrix (shared memory)
    lh_mat4 transform;  // the instance's
    MeshInfoRaster mi;
    uint32_t index_offset, triangle_offset;
    const Instance* inst;
};

// The warp's pass over one meshlet: its vertices transformed and snapped into
// shared memory, then one lane per triangle (set-up, face culling, binning).
// ALPHA: the alpha-clip class (double sided, alpha tested per fragment).
template <int KIND, bool ALPHA>
__device__ __forceinline__ void raster_meshlet(const FrameDev& f, const MeshletWork w, RasterTune tune, SnapV* sv,
                                               uint8_t* so, uint32_t* micro_words, AlphaVert* av, uint32_t lane,
                                               uint32_t& nfrag) {
    const uint32_t nv = w.nv, nt = w.nt, W = w.W, H = w.H;
    const MeshInfoRaster& mi = w.mi;
    AlphaSrc as{av, 0u, H};
    MeshInfoAlpha ma{};
    if (ALPHA) {
        ma = load_mesh_info_alpha(mesh_info_of(w.inst));
        as.tex = ma.tex;
    }
    // All of the meshlet's global loads are issued before any is used: the
    // micro-index words (at most 3 per lane; 4-byte aligned offsets, as the
    // meshletiser pads them), then both vertex indices of the lane, then both
    // positions -- two dependent round trips instead of seven.
    const uint64_t mbase = mi.micro_indices + w.triangle_offset;
    const uint32_t nbytes = nt * 3, nwords = (nbytes + 3) / 4;
    const bool micro_aligned = (mbase & 3) == 0;
    uint32_t mw[3] = {0u, 0u, 0u};
    if (micro_aligned) {
#pragma unroll
        for (uint32_t k = 0; k < 3; k++) {
            const uint32_t j = lane + 32u * k;
            if (j < nwords) mw[k] = __ldg(reinterpret_cast<const uint32_t*>(mbase) + j);
        }
    }
    const bool v0 = lane < nv, v1 = lane + 32u < nv;
    const uint32_t idx0 = v0 ? load_index_raw(mi.indices, mi.flags, w.index_offset + lane) : 0u;
    const uint32_t idx1 = v1 ? load_index_raw(mi.indices, mi.flags, w.index_offset + lane + 32u) : 0u;
    const f3 pos0 = v0 ? load_position(mi.positions, mi.flags, idx0) : f3{0.0f, 0.0f, 0.0f};
    const f3 pos1 = v1 ? load_position(mi.positions, mi.flags, idx1) : f3{0.0f, 0.0f, 0.0f};
    int32_t min_x = INT32_MAX, max_x = INT32_MIN, min_y = INT32_MAX, max_y = INT32_MIN;
    uint32_t any_oc = 0;
    auto vertex = [&](uint32_t j, uint32_t idx, f3 pos) {
        f3 wp = world_pos(w.transform, pos);
        f4 c = mul(*w.vp, f4{wp.x, wp.y, wp.z, 1.0f});
        uint32_t oc = outcode(c);
        SnapV s{0, 0, 0.0f};
        if (!oc) s = snap(c, w.hw, w.hh);
        sv[j] = s;
        so[j] = (uint8_t)oc;
        any_oc |= oc;
        min_x = min(min_x, s.X);
        max_x = max(max_x, s.X);
        min_y = min(min_y, s.Y);
        max_y = max(max_y, s.Y);
        if (ALPHA) av[j] = alpha_vert(c, ma, mi.flags, idx);
    };
    if (v0) vertex(lane, idx0, pos0);
    if (v1) vertex(lane + 32u, idx1, pos1);
    // A meshlet whose snapped vertices (all inside the guard band) span no
    // pixel centre produces no fragment: every triangle's bbox lies inside
    // the vertices' bbox.  Common for far meshlets in small views.
    if (nv > 0 && !__any_sync(0xFFFFFFFFu, any_oc != 0)) {
        min_x = __reduce_min_sync(0xFFFFFFFFu, min_x);
        max_x = __reduce_max_sync(0xFFFFFFFFu, max_x);
        min_y = __reduce_min_sync(0xFFFFFFFFu, min_y);
        max_y = __reduce_max_sync(0xFFFFFFFFu, max_y);
        if (max((min_x + 127) >> 8, 0) > min((max_x - 128) >> 8, (int32_t)W - 1) ||
            max((min_y + 127) >> 8, 0) > min((max_y - 128) >> 8, (int32_t)H - 1))
            return;
    }
    if (micro_aligned) {
#pragma unroll
        for (uint32_t k = 0; k < 3; k++) {
            const uint32_t j = lane + 32u * k;
            if (j < nwords) micro_words[j] = mw[k];
        }
    } else {
        uint8_t* d = reinterpret_cast<uint8_t*>(micro_words);
        for (uint32_t j = lane; j < nbytes; j += 32) d[j] = __ldg(reinterpret_cast<const uint8_t*>(mbase) + j);
    }
    __syncwarp();
    const uint8_t* mic = reinterpret_cast<const uint8_t*>(micro_words);
    for (uint32_t base = w.part * 32u; base < nt; base += 32u * w.split) {
        const uint32_t t = base + lane;
        bool medium = false, big = false;
        TriSetup st;
        if (t < nt) {
            const uint32_t m0 = mic[3 * t], m1 = mic[3 * t + 1], m2 = mic[3 * t + 2];
            if (m0 >= nv || m1 >= nv || m2 >= nv) {
                atomicOr(&f.status[kStFlags], LH_FLAG_BAD_MESHLET);
            } else {
                const uint32_t o0 = so[m0], o1 = so[m1], o2 = so[m2];
                if (((o0 | o1 | o2) & 64u) || (o0 & o1 & o2)) {
                    // non-finite / w <= 0, or entirely outside one plane
                } else if (o0 | o1 | o2) {
                    atomicAdd(&f.status[kStClipCount], 1u);  // statistics only
                    clip_triangle<KIND>(f, w.view, w.slot, t);
                } else {
                    SnapV a = sv[m0], b = sv[m1], c = sv[m2];
                    // most visible triangles hold no pixel centre: the 32-bit
                    // bbox test rejects them before the area.  The box and the
                    // area do not depend on the vertex order, so the set-up
                    // reuses both (make_setup's A is |cr| once oriented).
                    const TriBox box = tri_box(a, b, c, W, H);
                    int64_t cr = box_empty(box) ? 0 : cross_rel(a, b, c);
                    // alpha clip is double sided
                    bool keep = ALPHA ? cr != 0 : (KIND == 0 ? cr < 0 : cr > 0);
                    if (keep) {
                        if (cr > 0) { SnapV tmp = b; b = c; c = tmp; }
                        finish_setup(a, b, c, cr < 0 ? -cr : cr, box, LH_PACK_ID(t, w.slot), st);
                        if (ALPHA) {
                            st.bias |= kBiasAlpha;
                            st.verts = m0 | (m1 << 8) | (m2 << 16);
                        }
                        uint32_t npx = (uint32_t)(st.px1 - st.px0 + 1) * (uint32_t)(st.py1 - st.py0 + 1);
                        if (npx <= tune.small_px) {
                            if (ALPHA) nfrag += raster_lane_alpha<KIND>(f, st, w.target, W, as);
                            else raster_lane<KIND>(st, w.target, W, nfrag);
                        } else if (npx <= (KIND == 1 && LH_SHADOW_MEDIUM_PX ? min(tune.medium_px, (uint32_t)LH_SHADOW_MEDIUM_PX)
                                                                            : tune.medium_px)) {
                            medium = true;
                        } else {
                            big = true;  // appended below, one atomic per warp
                        }
                    }
                }
            }
        }
        // one atomic per warp on the queue's counter word: shadow views and
        // the occluder pass hold few meshlets with many big triangles each,
        // whose appends would otherwise queue on that one word
        if (__any_sync(0xFFFFFFFFu, big)) push_big_warp<KIND>(f, st, w.view, big, lane);
        uint32_t mask = __ballot_sync(0xFFFFFFFFu, medium);
        while (mask) {
            int src = __ffs(mask) - 1;
            mask &= mask - 1;
            TriSetup b = shfl_setup(st, src);
            if (ALPHA) nfrag += raster_warp_alpha<KIND>(f, b, w.target, W, lane, as);
            else raster_warp<KIND>(b, w.target, W, lane, nfrag);
        }
    }
    __syncwarp();
}

// Adds the warp's fragment count to the frame's statistics word of the
// pass (visibility or shadow views); called by every lane of the warp.
template <int KIND>
__device__ __forceinline__ void count_fragments(const FrameDev& f, uint32_t nfrag) {
    const uint32_t total = __reduce_add_sync(0xFFFFFFFFu, nfrag);
    if ((threadIdx.x & 31) == 0 && total) atomicAdd(&f.status[KIND == 0 ? kStFragVis : kStFragShadow], total);
}

// Meshlets of view `vw` a raster pass covers: every visible one of the class
// (kListAll), or the entries of one of the view's occlusion lists.
__device__ __forceinline__ uint32_t raster_list_count(const FrameDev& f, const ViewDev* vw, bool alpha, uint32_t list) {
    if (list == kListAll) return min(reinterpret_cast<const uint32_t*>(vw->draws)[alpha ? 1 : 0], f.max_draws);
    const uint32_t w = list == kListOccluders ? kClaimOccluders : (alpha ? kClaimSurvivorsAlpha : kClaimSurvivorsOpaque);
    return min(*reinterpret_cast<const volatile uint32_t*>(&vw->claim[w]), f.max_draws);
}
__device__ __forceinline__ uint32_t raster_list_slot(const FrameDev& f, const ViewDev* vw, bool alpha, uint32_t list,
                                                     uint32_t local) {
    if (list == kListAll) return alpha ? f.max_draws + local : local;
    const uint32_t k = list == kListOccluders ? 0u : (alpha ? 2u : 1u);
    return __ldcg(vw->lists + (size_t)k * f.max_draws + local);
}

// One warp per visible meshlet of views [view_begin, view_begin + n_views)
// of one draw class (opaque, or ALPHA: alpha clip), claimed from
// `claim_word`; `list` selects all of them or one occlusion list.
// Persistent: returns when the claims run out.  The classes are separate
// instantiations (separate launches) so that the opaque path carries none
// of the alpha test's state.
template <int KIND, bool ALPHA>
__device__ void phase_raster(const FrameDev& f, uint32_t view_begin, uint32_t n_views, RasterTune tune,
                             uint32_t* claim_word, RasterSmem& sm, AlphaVert (*s_av)[MAX_MESHLET_UNIQUE_VERTICES],
                             uint32_t list = kListAll) {
    uint32_t* s_prefix = sm.prefix;
    lh_mat4* s_vp = sm.vp;
    SnapV(*s_v)[MAX_MESHLET_UNIQUE_VERTICES] = sm.v;
    uint8_t(*s_oc)[MAX_MESHLET_UNIQUE_VERTICES] = sm.oc;
    uint32_t(*s_micro)[kMicroWords] = sm.micro;
    __syncthreads();  // `sm` may still be in use by a previous phase of the block
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t v = 0; v < n_views; v++) {
            s_prefix[v] = run;
            run += raster_list_count(f, f.views + view_begin + v, ALPHA, list);
        }
        s_prefix[n_views] = run;
    }
    for (uint32_t i = threadIdx.x; i < n_views * 16; i += blockDim.x) {
        const lh_mat4& m = view_matrix(f, f.views + view_begin + i / 16);
        reinterpret_cast<float*>(&s_vp[i / 16])[i % 16] = reinterpret_cast<const float*>(&m)[i % 16];
    }
    __syncthreads();
    const uint32_t total = s_prefix[n_views];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    SnapV* sv = s_v[warp];
    uint8_t* so = s_oc[warp];
    // Work units: a meshlet, or a quarter of its triangles when the views
    // hold fewer than two meshlets per warp of the grid (shadow cascades).
    // Units are claimed `batch` per atomic: one keeps consecutive (nearby)
    // meshlets on different warps; with millions of units (many views) the
    // claim word itself becomes the contended address and 4 pays.
    const uint32_t warps_total = gridDim.x * (blockDim.x >> 5);
    const uint32_t split = total < 2u * warps_total ? 4u : 1u;
    const uint32_t units = total * split;
    const uint32_t batch = tune.batch ? tune.batch : (units > 256u * warps_total ? 4u : 1u);
    // The first window of every warp is static (warp g takes units
    // [g * batch, (g + 1) * batch)); the claim word hands out the rest from
    // warps_total * batch on.  Launches with fewer units than warps (shadow
    // cascades) then touch the claim word not at all, and none start with
    // every warp queueing on it.
    const uint32_t gwarp = blockIdx.x * (blockDim.x >> 5) + warp;
    const uint32_t dyn_base = warps_total * batch;
    uint32_t unit = min(gwarp * batch, units), unit_end = min(gwarp * batch + batch, units);
    // Each claim is issued when the window before it starts, so the atomic's
    // round trip overlaps that window's work (a warp holds at most one
    // window it has not started).
    const bool dynamic = dyn_base < units;
    uint32_t pending = 0;
    if (dynamic && lane == 0) pending = atomicAdd(claim_word, batch);
    // A warp's units only increase (its static window, then claims that
    // increase over time), so the view search starts at the previous unit's
    // view: with many views (probes) a search from view 0 is a chain of
    // dependent shared-memory loads per unit.
    uint32_t v = 0;
    uint32_t nfrag = 0;  // fragments this lane wrote
    for (;;) {
        if (unit >= unit_end) {
            if (!dynamic) break;
            const uint32_t first = dyn_base + __shfl_sync(0xFFFFFFFFu, pending, 0);
            if (first >= units) break;
            unit = first;
            unit_end = min(first + batch, units);
            if (lane == 0) pending = atomicAdd(claim_word, batch);
        }
        const uint32_t item = unit / split, part = unit % split;
        unit++;
        if (item < s_prefix[v]) v = 0;  // not expected; keeps the search exact regardless
        while (item >= s_prefix[v + 1]) v++;
        const uint32_t view = view_begin + v;
        const ViewDev* vw = f.views + view;
        const uint32_t local = item - s_prefix[v];
        const uint32_t slot = raster_list_slot(f, vw, ALPHA, list, local);
        // the slot's draw record (written by the meshlet cull): the index and
        // micro-index addresses come offset to the meshlet already
        const RasterDraw rd = vw->rdraws[slot];
        const Instance* inst = f.instances + rd.instance;
        lh_mat4 transform;
        load_transform(inst, transform);
        MeshInfoRaster mi;
        mi.positions = rd.positions;
        mi.indices = rd.indices;
        mi.micro_indices = rd.micro;
        mi.meshlets = 0;
        mi.flags = rd.bits >> 16;
        const uint32_t W = vw->width, H = vw->height;
        void* target = vw->target;
        const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
        const uint32_t nv = rd.bits & 0xFFu, nt = (rd.bits >> 8) & 0xFFu;
        if (nv > MAX_MESHLET_UNIQUE_VERTICES || nt > MAX_MESHLET_TRIANGLES) {
            // beyond the meshletiser limits: malformed, skipped and flagged
            if (lane == 0 && part == 0) atomicOr(&f.status[kStFlags], LH_FLAG_BAD_MESHLET);
            continue;
        }
        if (part * 32u >= nt) continue;  // this quarter holds no triangles
        if (rd.bits & kDrawNoCentre) continue;  // no pixel centre in reach of its sphere
        const MeshletWork w{view, slot, part, split, nv, nt, W, H, target, hw, hh, &s_vp[v], transform, mi, 0u, 0u, inst};
        raster_meshlet<KIND, ALPHA>(f, w, tune, sv, so, s_micro[warp], ALPHA ? s_av[warp] : nullptr, lane, nfrag);
    }
    count_fragments<KIND>(f, nfrag);
}

// Edge function of edge a->b at pixel centre (px, py).
__device__ __forceinline__ int64_t edge_at(int32_t ax, int32_t ay, int32_t bx, int32_t by, int32_t px, int32_t py) {
    return (int64_t)(by - ay) * ((int64_t)px * 256 + 128 - ax) - (int64_t)(bx - ax) * ((int64_t)py * 256 + 128 - ay);
}

// True when the edge's test fails at all four corners of the pixel
// rectangle (the edge function is affine, so it fails everywhere inside).
__device__ __forceinline__ bool edge_rejects(int32_t ax, int32_t ay, int32_t bx, int32_t by, int32_t x0, int32_t x1,
                                             int32_t y0, int32_t y1, int64_t bias) {
    return edge_at(ax, ay, bx, by, x0, y0) < bias && edge_at(ax, ay, bx, by, x1, y0) < bias &&
           edge_at(ax, ay, bx, by, x0, y1) < bias && edge_at(ax, ay, bx, by, x1, y1) < bias;
}

// Edge values of a chunk's covered pixels, by the triangle's doubled area
// 2A (= e12 + e20 + e01 at every point, so no covered pixel's value exceeds
// it): kEdge32 below 2^31 (32-bit arithmetic, exact modulo 2^32 and so
// exact for these values; the 32-bit conversion instruction), kEdge46 below
// 2^46 (64-bit, FP32-add conversion), kEdge64 beyond (the 64-bit conversion
// instruction).
enum EdgeMode { kEdge32 = 0, kEdge46 = 1, kEdge64 = 2 };
template <int MODE>
struct EdgeVal {
    using T = typename std::conditional<MODE == kEdge32, uint32_t, int64_t>::type;
};
template <int MODE>
__device__ __forceinline__ float covered_to_float(typename EdgeVal<MODE>::T v) {
    if (MODE == kEdge32) return __uint2float_rn((uint32_t)v);
    if (MODE == kEdge46) return u46_to_f32_rn((uint64_t)v);
    return __ll2float_rn((int64_t)v);
}
template <int MODE>
__device__ __forceinline__ typename EdgeVal<MODE>::T shfl_edge(typename EdgeVal<MODE>::T v, uint32_t src) {
    if (MODE == kEdge32) return (uint32_t)__shfl_sync(0xFFFFFFFFu, (uint32_t)v, src);
    return (int64_t)__shfl_sync(0xFFFFFFFFu, (unsigned long long)v, src);
}

// The triangle's depth plane and ID, held in registers during a walk.
struct ChunkDepth {
    float z0, s1, s2;
    uint32_t id;
};

// A covered pixel: depth from its two edge values (the per-pixel test's
// arithmetic), then the depth test at linear pixel index `pix`.
template <int KIND, int MODE>
__device__ __forceinline__ void chunk_fragment(const ChunkDepth& t, void* target, uint32_t pix,
                                               typename EdgeVal<MODE>::T a20, typename EdgeVal<MODE>::T a01) {
    float d = (t.z0 + covered_to_float<MODE>(a20) * t.s1) + covered_to_float<MODE>(a01) * t.s2;
    d = d > 0.0f ? d : 0.0f;
    d = d < 1.0f ? d : 1.0f;
    if (KIND == 0) {
        const unsigned long long key = ((unsigned long long)f2u(d) << 32) | t.id;
        asm volatile("red.relaxed.gpu.global.max.u64 [%0], %1;" ::"l"(reinterpret_cast<unsigned long long*>(target) + pix),
                     "l"(key));
    } else {
        asm volatile("red.relaxed.gpu.global.min.u32 [%0], %1;" ::"l"(reinterpret_cast<uint32_t*>(target) + pix),
                     "r"(f2u(d)));
    }
}

// Row by row: the warp's lanes along each run (long runs).  Lane r holds
// row r's run: its length, the linear index of its first pixel and the two
// edge values there.
template <int KIND, int MODE>
__device__ __forceinline__ uint32_t chunk_rows(const ChunkDepth& t, void* target, uint32_t rows, uint32_t lane,
                                               int32_t len, uint32_t pix_first, typename EdgeVal<MODE>::T f20,
                                               typename EdgeVal<MODE>::T f01, typename EdgeVal<MODE>::T dx20,
                                               typename EdgeVal<MODE>::T dx01) {
    using T = typename EdgeVal<MODE>::T;
    uint32_t nfrag = 0;
    const T step20 = 32 * dx20, step01 = 32 * dx01;
    for (uint32_t r = 0; r < rows; r++) {
        const int32_t l = __shfl_sync(0xFFFFFFFFu, len, r);
        if (l == 0) continue;
        uint32_t pix = __shfl_sync(0xFFFFFFFFu, pix_first, r) + lane;
        T a20 = shfl_edge<MODE>(f20, r) + (T)lane * dx20, a01 = shfl_edge<MODE>(f01, r) + (T)lane * dx01;
        for (int32_t k = (int32_t)lane; k < l; k += 32, pix += 32, a20 += step20, a01 += step01) {
            chunk_fragment<KIND, MODE>(t, target, pix, a20, a01);
            nfrag++;
        }
    }
    return nfrag;
}

// Compacted: the covered pixels of all rows numbered one after another,
// 32 consecutive per step, one per lane (short runs: slivers, corners).
// The non-empty rows are ranked in row order and lane k holds the k-th
// one's run: its first number, and the linear index and edge values
// extrapolated to number 0.  A step over numbers [base, base + 32) marks
// the runs that start inside it in one word (a warp OR of one bit per
// run), so a lane's run is the last one started at or before its number:
// the runs started before the step plus those marked up to its own bit.
template <int KIND, int MODE>
__device__ __forceinline__ uint32_t chunk_compact(const ChunkDepth& t, void* target, uint32_t lane, int32_t total,
                                                  int32_t first, uint32_t pix_zero, typename EdgeVal<MODE>::T z20,
                                                  typename EdgeVal<MODE>::T z01, typename EdgeVal<MODE>::T dx20,
                                                  typename EdgeVal<MODE>::T dx01, uint32_t nonempty) {
    using T = typename EdgeVal<MODE>::T;
    uint32_t nfrag = 0;
    const uint32_t upto_me = 0xFFFFFFFFu >> (31u - lane);  // bits 0 .. lane
    int32_t before = 0;  // runs started before the step
    for (int32_t base = 0; base < total; base += 32) {
        const uint32_t off = (uint32_t)(first - base);
        const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, lane < nonempty && off < 32u ? 1u << off : 0u);
        const int32_t k = before + __popc(starts & upto_me) - 1;  // the lane's run
        before += __popc(starts);
        const int32_t p = base + (int32_t)lane;
        const uint32_t src = (uint32_t)k & 31u;
        const uint32_t pix = (uint32_t)p + __shfl_sync(0xFFFFFFFFu, pix_zero, src);
        const T a20 = shfl_edge<MODE>(z20, src) + (T)p * dx20, a01 = shfl_edge<MODE>(z01, src) + (T)p * dx01;
        if (p < total) {
            chunk_fragment<KIND, MODE>(t, target, pix, a20, a01);
            nfrag++;
        }
    }
    return nfrag;
}

// Per-row run state of a chunk, then the cheaper of the two walks.
template <int KIND, int MODE>
__device__ __forceinline__ uint32_t chunk_walk(const BigTri& b, void* target, uint32_t W, int32_t x0, int32_t y0,
                                               uint32_t rows, uint32_t lane, int32_t lo, int32_t len, int32_t pre,
                                               int32_t total, int64_t e20, int64_t e01, int64_t dx20, int64_t dx01) {
    using T = typename EdgeVal<MODE>::T;
    const ChunkDepth t{b.z0, b.s1, b.s2, b.id};
    // steps of the row walk (plus a row's own cost) against the compacted
    // walk's, whose steps cost about twice as much
    const uint32_t row_steps = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)(len + 31) >> 5);
    const uint32_t ne_mask = __ballot_sync(0xFFFFFFFFu, len > 0);
    const uint32_t nonempty = __popc(ne_mask);
    const uint32_t pix_row = (uint32_t)(y0 + (int32_t)lane) * W + (uint32_t)x0;
    if (row_steps + nonempty / 4u <= 2u * (uint32_t)((total + 31) >> 5))
        return chunk_rows<KIND, MODE>(t, target, rows, lane, len, pix_row + (uint32_t)lo, (T)(e20 + (int64_t)lo * dx20),
                                      (T)(e01 + (int64_t)lo * dx01), (T)dx20, (T)dx01);
    // rank the non-empty rows: lane k takes the k-th one's values
    const uint32_t src = __fns(ne_mask, 0, (int32_t)lane + 1);  // 0xFFFFFFFF past the last
    const uint32_t s = src < 32u ? src : 0u;
    const int32_t first = __shfl_sync(0xFFFFFFFFu, pre, s);
    const uint32_t pix_zero = __shfl_sync(0xFFFFFFFFu, pix_row + (uint32_t)(lo - pre), s);
    const T z20 = shfl_edge<MODE>((T)(e20 + (int64_t)(lo - pre) * dx20), s);
    const T z01 = shfl_edge<MODE>((T)(e01 + (int64_t)(lo - pre) * dx01), s);
    return chunk_compact<KIND, MODE>(t, target, lane, total, first, pix_zero, z20, z01, (T)dx20, (T)dx01, nonempty);
}

// The pixels [x0, x1] x [y0, y1] (at most 32 rows of at most 256) of an
// opaque big triangle, by the whole warp.  Lane r finds the run of covered
// pixels of row y0 + r (the three edges' runs intersected, clip_run); the
// runs are walked row by row when they are long, else compacted (every lane
// of a step on a covered pixel).  Either walk forms, at every pixel, the
// very integers the per-pixel test forms, so coverage and depth are the
// same; a step's pixels lie in one or two rows, so its reductions stay
// coalesced.  Returns the fragments written.
struct ChunkSteps {  // a triangle's edge steps along x and their reciprocals
    int64_t dx12, dx20, dx01;
    float inv12, inv20, inv01;
};
__device__ __forceinline__ ChunkSteps chunk_steps(const BigTri& b) {
    ChunkSteps k;
    k.dx12 = (int64_t)(b.Y2 - b.Y1) * 256;
    k.dx20 = (int64_t)(b.Y0 - b.Y2) * 256;
    k.dx01 = (int64_t)(b.Y1 - b.Y0) * 256;
    k.inv12 = run_inv_step(b.Y2 - b.Y1);
    k.inv20 = run_inv_step(b.Y0 - b.Y2);
    k.inv01 = run_inv_step(b.Y1 - b.Y0);
    return k;
}

template <int KIND>
__device__ __forceinline__ uint32_t raster_chunk_runs(const BigTri& b, const ChunkSteps& k, int32_t x0, int32_t x1,
                                                      int32_t y0, int32_t y1, uint32_t lane, void* target, uint32_t W) {
    const int32_t n = x1 - x0 + 1;
    const uint32_t rows = (uint32_t)(y1 - y0 + 1);
    const int64_t dx20 = k.dx20, dx01 = k.dx01;
    int32_t lo = 0, hi = -1;
    int64_t e12 = 0, e20 = 0, e01 = 0;
    if (lane < rows) {
        const int32_t y = y0 + (int32_t)lane;
        e12 = edge_at(b.X1, b.Y1, b.X2, b.Y2, x0, y);
        e20 = edge_at(b.X2, b.Y2, b.X0, b.Y0, x0, y);
        e01 = edge_at(b.X0, b.Y0, b.X1, b.Y1, x0, y);
        hi = n - 1;
        clip_run(e12, k.dx12, b.bias & 1u, n, k.inv12, lo, hi);
        clip_run(e20, dx20, (b.bias >> 1) & 1u, n, k.inv20, lo, hi);
        clip_run(e01, dx01, (b.bias >> 2) & 1u, n, k.inv01, lo, hi);
    }
    const int32_t len = hi >= lo ? hi - lo + 1 : 0;
    int32_t incl = len;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    const int32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total == 0) return 0;
    const int32_t pre = incl - len;
    // 2A: the sum of the three edge functions, the same at every point
    const uint64_t area2 = (uint64_t)__shfl_sync(0xFFFFFFFFu, (unsigned long long)(e12 + e20 + e01), 0);
    if (area2 < (1ull << 31))
        return chunk_walk<KIND, kEdge32>(b, target, W, x0, y0, rows, lane, lo, len, pre, total, e20, e01, dx20, dx01);
    if (area2 < (1ull << 46))
        return chunk_walk<KIND, kEdge46>(b, target, W, x0, y0, rows, lane, lo, len, pre, total, e20, e01, dx20, dx01);
    return chunk_walk<KIND, kEdge64>(b, target, W, x0, y0, rows, lane, lo, len, pre, total, e20, e01, dx20, dx01);
}

// Number of entries of the ascending array base[0, n) that are <= c (the
// upper bound), found by the whole warp: 32 probes per round narrow the
// range 32-fold, so a queue of 16k triangles takes 3 dependent loads instead
// of 14.
__device__ __forceinline__ uint32_t upper_bound_warp(const uint32_t* base, uint32_t n, uint32_t c, uint32_t lane) {
    uint32_t lo = 0, hi = n;  // the answer lies in [lo, hi]
    for (;;) {
        const uint32_t span = hi - lo;
        const uint32_t step = span <= 32u ? 1u : (span + 31u) / 32u;
        const uint32_t p = lo + lane * step;
        const bool le = p < hi && __ldcg(base + p) <= c;
        const uint32_t k = __popc(__ballot_sync(0xFFFFFFFFu, le));  // true lanes form a prefix
        if (step == 1u) return lo + k;
        const uint32_t nlo = k ? lo + (k - 1u) * step + 1u : lo;
        const uint32_t nhi = (k < 32u && lo + k * step < hi) ? lo + k * step : hi;
        lo = nlo;
        hi = nhi;
    }
}

// The pixels [x0, x1] x [y0, y1] of an alpha-tested big triangle, one
// column per lane (not inlined, as the other alpha paths).  The triangle is
// passed as its queue entry: a reference to the caller's copy would keep
// that copy in local memory on the opaque path too.
template <int KIND>
__device__ __noinline__ uint32_t raster_chunk_alpha(const FrameDev& f, const BigTri* entry, int32_t x0, int32_t x1,
                                                    int32_t y0, int32_t y1, uint32_t lane) {
    const BigTri b = *entry;
    const ViewDev* vw = f.views + b.view;
    void* target = vw->target;
    const uint32_t W = vw->width, H = vw->height;
    const AlphaTri at = alpha_tri_global(f, b.view, b.id);
    TriSetup t;
    t.X0 = b.X0; t.Y0 = b.Y0; t.X1 = b.X1; t.Y1 = b.Y1; t.X2 = b.X2; t.Y2 = b.Y2;
    t.z0 = b.z0; t.s1 = b.s1; t.s2 = b.s2;
    t.id = b.id;
    t.bias = b.bias;
    uint32_t n = 0;
    for (int32_t py = y0; py <= y1; py++)
        for (int32_t px = x0 + (int32_t)lane; px <= x1; px += 32) {
            float d;
            if (cover(t, px, py, d) && alpha_pass(f, at, px, py, W, H)) {
                write_fragment<KIND>(target, W, px, py, d, t.id);
                n++;
            }
        }
    return n;
}

// One warp per chunk of a big triangle (rows x columns of f.chunk_shift,
// at most 32 x 256 pixels): opaque chunks by runs of covered pixels
// (raster_chunk_runs), alpha-tested ones pixel by pixel, skipped whole when
// their rectangle lies outside one edge.
// Asynchronous 16-byte copy global -> shared through L2 (cp.async.cg), and
// the wait for the issuing thread's copies.
__device__ __forceinline__ void cp_async16_cg(void* smem, const void* gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int KIND>
__device__ void phase_raster_big(const FrameDev& f) {
    // the views' targets and widths, read once per block
    __shared__ unsigned long long s_target[kMaxViews];
    __shared__ uint32_t s_width[kMaxViews];
    // each warp's current triangle and the queue's next one (copied ahead
    // with cp.async while the current one's chunks are walked), kept in
    // shared memory, not registers; blocks of kRasterWarps warps
    __shared__ __align__(16) BigTri s_tri[kRasterWarps][2];
    __shared__ ChunkSteps s_steps[kRasterWarps];
    __syncthreads();  // a previous call of this phase in the block may still read them
    for (uint32_t v = threadIdx.x; v < f.n_views; v += blockDim.x) {
        s_target[v] = reinterpret_cast<unsigned long long>(f.views[v].target);
        s_width[v] = f.views[v].width;
    }
    __syncthreads();
    const unsigned long long packed = *reinterpret_cast<volatile unsigned long long*>(f.status + kStBigPacked);
    const uint32_t ntri = (uint32_t)min((unsigned long long)f.big_cap, packed >> 40);
    const unsigned long long total = packed & ((1ull << 40) - 1);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (ntri == 0) return;
    // chunk numbers fit 32 bits (push_big drops triangles beyond)
    const uint32_t total32 = (uint32_t)min(total, 0xFFFFFFFFull);
    // static first batch per warp, then claims from warps * kChunkBatch on;
    // chunks claimed per atomic: LH_CHUNK_BATCH, or 16 when the queue holds
    // more than 256 chunks per warp (millions of chunks would otherwise
    // queue on the one claim word)
    const uint32_t warps_total = gridDim.x * (blockDim.x >> 5);
    const uint32_t kChunkBatch = total32 > 256u * warps_total ? 16u : (uint32_t)LH_CHUNK_BATCH;
    const uint32_t gwarp = blockIdx.x * (blockDim.x >> 5) + w;
    const uint64_t dyn_base = (uint64_t)warps_total * kChunkBatch;
    const uint32_t rs = f.chunk_shift[KIND][0], cs = f.chunk_shift[KIND][1];
    uint32_t c = (uint32_t)min((uint64_t)gwarp * kChunkBatch, (uint64_t)total32);
    uint32_t c_end = (uint32_t)min((uint64_t)gwarp * kChunkBatch + kChunkBatch, (uint64_t)total32);
    // the current triangle, kept while consecutive chunks belong to it:
    // its entry, chunk range [t_base, t_end), chunk columns, shared-memory
    // slot, and the coordinates of the last chunk taken (number c_last);
    // the copied-ahead next entry (index pre_idx, chunk range [pb1, pb2))
    uint32_t t_idx = 0, t_base = 1, t_end = 0, nbx = 1, c_last = 0xFFFFFFFFu, slot = 0;
    uint32_t pre_idx = 0xFFFFFFFFu, pb1 = 0, pb2 = 0;
    int32_t cx = 0, cy = 0;
    const ChunkSteps& ks = s_steps[w];
    uint32_t nfrag = 0;
    for (;;) {
        if (c >= c_end) {
            if (dyn_base >= total32) break;
            uint32_t first_c = 0;
            if (lane == 0) first_c = atomicAdd(&f.status[kStBigClaim], kChunkBatch);
            first_c = __shfl_sync(0xFFFFFFFFu, first_c, 0);
            const uint64_t first = dyn_base + first_c;
            if (first >= total32) break;
            c = (uint32_t)first;
            c_end = (uint32_t)min(first + kChunkBatch, (uint64_t)total32);
        }
        if (c >= t_base && c < t_end) {
            // the same triangle: the next chunk in row order, or any other
            if (c == c_last + 1u) {
                if (++cx == (int32_t)nbx) {
                    cx = 0;
                    cy++;
                }
            } else {
                cx = (int32_t)((c - t_base) % nbx);
                cy = (int32_t)((c - t_base) / nbx);
            }
        } else {
            // another triangle: the copied-ahead next entry when c lies in
            // its range (chunk numbers ascend with the entries), else a
            // 32-ary search of the bases and a load
            __syncwarp();  // every lane is done with the current slot
            uint32_t i, base;
            if (pre_idx != 0xFFFFFFFFu && c >= pb1 && c < pb2) {
                i = pre_idx;
                base = pb1;
                cp_async_wait_all();
                __syncwarp();
                slot ^= 1u;
            } else {
                const uint32_t first = upper_bound_warp(f.big_base, ntri, c, lane);
                if (first == 0) {
                    c++;
                    continue;
                }
                i = first - 1;
                const BigTri nb = f.big[i];
                base = f.big_base[i];
                if (lane == 0) s_tri[w][slot] = nb;
                __syncwarp();
            }
            const BigTri& nb = s_tri[w][slot];
            const uint32_t nx = ((uint32_t)(nb.px1 - nb.px0) >> cs) + 1;
            const uint32_t ny = ((uint32_t)(nb.py1 - nb.py0) >> rs) + 1;
            if ((unsigned long long)(c - base) >= (unsigned long long)nx * ny) {  // chunk of a dropped triangle
                t_base = 1;  // the slot no longer holds the current triangle
                t_end = 0;
                pre_idx = 0xFFFFFFFFu;
                c++;
                continue;
            }
            if (lane == 0) s_steps[w] = chunk_steps(nb);
            t_idx = i;
            t_base = base;
            t_end = base + nx * ny;
            nbx = nx;
            cx = (int32_t)((c - base) % nx);
            cy = (int32_t)((c - base) / nx);
            // copy the queue's next entry into the other slot meanwhile
            pre_idx = 0xFFFFFFFFu;
            if (i + 1u < ntri) {
                if (lane < 4) {
                    cp_async_wait_all();  // a copy still in flight to that slot
                    cp_async16_cg(reinterpret_cast<char*>(&s_tri[w][slot ^ 1u]) + 16 * lane,
                                  reinterpret_cast<const char*>(f.big + i + 1u) + 16 * lane);
                    cp_async_commit();
                }
                pb1 = f.big_base[i + 1u];
                pb2 = i + 2u < ntri ? f.big_base[i + 2u] : total32;
                pre_idx = i + 1u;
            }
            __syncwarp();
        }
        c_last = c;
        c++;
        const BigTri& b = s_tri[w][slot];
        const int32_t x0 = b.px0 + (cx << cs), x1 = min(b.px1, x0 + (1 << cs) - 1);
        const int32_t y0 = b.py0 + (cy << rs), y1 = min(b.py1, y0 + (1 << rs) - 1);
        void* target = reinterpret_cast<void*>(s_target[b.view]);
        const uint32_t W = s_width[b.view];
        if (b.bias & kBiasAlpha) {
            if (edge_rejects(b.X1, b.Y1, b.X2, b.Y2, x0, x1, y0, y1, b.bias & 1u) ||
                edge_rejects(b.X2, b.Y2, b.X0, b.Y0, x0, x1, y0, y1, (b.bias >> 1) & 1u) ||
                edge_rejects(b.X0, b.Y0, b.X1, b.Y1, x0, x1, y0, y1, (b.bias >> 2) & 1u))
                continue;
            nfrag += raster_chunk_alpha<KIND>(f, f.big + t_idx, x0, x1, y0, y1, lane);
            continue;
        }
        nfrag += raster_chunk_runs<KIND>(b, ks, x0, x1, y0, y1, lane, target, W);
    }
    cp_async_wait_all();  // no copy outlives the phase
    count_fragments<KIND>(f, nfrag);
}

// ------------------------------------------------------------ occlusion
// Hierarchical depth of the visibility views [view_begin, view_begin +
// n_views) that cull by occlusion, after the occluder pass: one block of 256
// threads per 64 x 64-pixel region (regions of all these views numbered one
// after another), claimed round robin by the grid.  Warp w takes pixel rows
// 8w .. 8w + 7 of the region in two 32-pixel halves, keeps the minimum depth
// bits of each lane's column, then of each 8 x 8 tile (lanes in groups of
// 8); the block takes the region's minimum over its 64 tiles.  Pixels
// outside the view do not count; a pixel without a fragment is depth 0.
__device__ void phase_hiz(const FrameDev& f, uint32_t view_begin, uint32_t n_views) {
    __shared__ uint32_t s_region_min[8];
    __shared__ uint32_t s_first[kMaxViews + 1];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();  // shared memory may still be in use by a previous phase of the block
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t v = 0; v < n_views; v++) {
            const ViewDev* vw = f.views + view_begin + v;
            s_first[v] = run;
            if (vw->kind == kViewVisibility && vw->hiz) run += vw->hiz_rx * vw->hiz_ry;
        }
        s_first[n_views] = run;
    }
    __syncthreads();
    const uint32_t total = s_first[n_views];
    uint32_t v = 0;
    for (uint32_t region = blockIdx.x; region < total; region += gridDim.x) {
        while (region >= s_first[v + 1]) v++;
        const ViewDev* vw = f.views + view_begin + v;
        const uint32_t r = region - s_first[v], rx = r % vw->hiz_rx, ry = r / vw->hiz_rx;
        const uint32_t W = vw->width, H = vw->height;
        const uint64_t* vis = reinterpret_cast<const uint64_t*>(vw->target);
        uint32_t* level0 = vw->hiz;
        const uint32_t pitch0 = vw->hiz_rx * 8u;
        uint32_t wmin = 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            const uint32_t x = rx * kHizRegion + half * 32u + lane;
            uint32_t m = 0xFFFFFFFFu;
#pragma unroll
            for (uint32_t k = 0; k < 8; k++) {
                const uint32_t y = ry * kHizRegion + warp * 8u + k;
                if (x < W && y < H) m = min(m, (uint32_t)(__ldcg(vis + (size_t)y * W + x) >> 32));
            }
            m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, 1));
            m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, 2));
            m = min(m, __shfl_xor_sync(0xFFFFFFFFu, m, 4));
            if ((lane & 7u) == 0) level0[(size_t)(ry * 8u + warp) * pitch0 + rx * 8u + half * 4u + (lane >> 3)] = m;
            wmin = min(wmin, m);
        }
        wmin = __reduce_min_sync(0xFFFFFFFFu, wmin);
        if (lane == 0) s_region_min[warp] = wmin;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t m = s_region_min[0];
            for (uint32_t k = 1; k < 8; k++) m = min(m, s_region_min[k]);
            level0[(size_t)pitch0 * vw->hiz_ry * 8u + r] = m;  // level 1
        }
        __syncthreads();
    }
}

// True when no fragment of a meshlet inside the world sphere `sp` can pass
// the depth test against what the view holds already: every 8 x 8 tile (or
// 64 x 64 region) its screen box touches has a minimum depth above the
// largest depth the sphere can reach.  The box and that depth come from the
// 8 corners of the sphere's axis-aligned box through the view's matrix,
// widened by 2 pixels and by 1/128 of the depth (the kernels' float
// rounding of the vertices is far below both); a corner at or behind the
// camera plane culls nothing.  Exact: a culled meshlet's every fragment
// would have lost the atomicMax (its depth strictly below the pixel's).
__device__ __forceinline__ bool hiz_occluded(const ViewDev* vw, const lh_mat4& pv, const float (&sp)[4]) {
    const f4 cc = mul(pv, f4{sp[0], sp[1], sp[2], 1.0f});
    const float r = sp[3];
    const f4 a{pv.cols[0].x * r, pv.cols[0].y * r, pv.cols[0].z * r, pv.cols[0].w * r};
    const f4 b{pv.cols[1].x * r, pv.cols[1].y * r, pv.cols[1].z * r, pv.cols[1].w * r};
    const f4 d{pv.cols[2].x * r, pv.cols[2].y * r, pv.cols[2].z * r, pv.cols[2].w * r};
    const float hw = (float)vw->width * 0.5f, hh = (float)vw->height * 0.5f;
    float x0 = 3.0e38f, x1 = -3.0e38f, y0 = 3.0e38f, y1 = -3.0e38f, zmax = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float sa = (k & 1) ? 1.0f : -1.0f, sb = (k & 2) ? 1.0f : -1.0f, sd = (k & 4) ? 1.0f : -1.0f;
        const float cw = cc.w + sa * a.w + sb * b.w + sd * d.w;
        if (!(cw > 1e-6f)) return false;
        const float cx = cc.x + sa * a.x + sb * b.x + sd * d.x;
        const float cy = cc.y + sa * a.y + sb * b.y + sd * d.y;
        const float cz = cc.z + sa * a.z + sb * b.z + sd * d.z;
        const float px = (cx / cw) * hw + hw, py = (cy / cw) * hh + hh, pz = cz / cw;
        x0 = fminf(x0, px);
        x1 = fmaxf(x1, px);
        y0 = fminf(y0, py);
        y1 = fmaxf(y1, py);
        zmax = fmaxf(zmax, pz);
    }
    if (!(zmax >= 0.0f) || !(x1 >= x0) || !(y1 >= y0)) return false;  // NaN
    const float zt = zmax + zmax * (1.0f / 128.0f);
    if (!(zt < 1.0f)) return false;
    const uint32_t zbits = __float_as_uint(zt);
    const int32_t W = (int32_t)vw->width, H = (int32_t)vw->height;
    // the box, widened and clamped to [-1, W] x [-1, H] before conversion
    auto px_lo = [](float v, float lim) { return fminf(fmaxf(floorf(v) - 2.0f, -1.0f), lim); };
    auto px_hi = [](float v, float lim) { return fminf(fmaxf(ceilf(v) + 2.0f, -1.0f), lim); };
    const int32_t ix0 = max((int32_t)px_lo(x0, (float)W), 0), ix1 = min((int32_t)px_hi(x1, (float)W), W - 1);
    const int32_t iy0 = max((int32_t)px_lo(y0, (float)H), 0), iy1 = min((int32_t)px_hi(y1, (float)H), H - 1);
    if (ix0 > ix1 || iy0 > iy1) return true;  // no pixel centre of the view in reach
    const uint32_t pitch0 = vw->hiz_rx * 8u;
    const uint32_t* level0 = vw->hiz;
    // the ≤ 16 tiles (or regions) under the box, loaded all at once (no
    // load waits on the previous one's compare), then their minimum
    auto box_min = [](const uint32_t* level, uint32_t pitch, int32_t tx0, int32_t tx1, int32_t ty0, int32_t ty1) {
        const int32_t n = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
        uint32_t m = 0xFFFFFFFFu;
        int32_t tx = tx0, ty = ty0;
#pragma unroll
        for (int32_t k = 0; k < 16; k++) {
            if (k < n) {
                m = min(m, __ldcg(level + (size_t)ty * pitch + tx));
                if (++tx > tx1) {
                    tx = tx0;
                    ty++;
                }
            }
        }
        return m;
    };
    int32_t tx0 = ix0 >> 3, tx1 = ix1 >> 3, ty0 = iy0 >> 3, ty1 = iy1 >> 3;
    if ((tx1 - tx0 + 1) * (ty1 - ty0 + 1) <= 16) return box_min(level0, pitch0, tx0, tx1, ty0, ty1) > zbits;
    const uint32_t* level1 = level0 + (size_t)pitch0 * vw->hiz_ry * 8u;
    tx0 = ix0 >> 6, tx1 = ix1 >> 6, ty0 = iy0 >> 6, ty1 = iy1 >> 6;
    if ((tx1 - tx0 + 1) * (ty1 - ty0 + 1) > 16) return false;
    return box_min(level1, vw->hiz_rx, tx0, tx1, ty0, ty1) > zbits;
}

// After the hierarchical depth: every visible meshlet of the visibility
// views that is not an occluder (opaque, then alpha clip) is tested against
// it, and the survivors go to the view's survivor lists for the second
// raster pass (warp-aggregated appends, any order).  Threads stride over
// the (view, meshlet) pairs.  Also resets the raster's claim and big-triangle
// words for that pass (nothing of the occluder pass runs any more).
__device__ void phase_occlusion_filter(const FrameDev& f, uint32_t view_begin, uint32_t n_views, uint64_t gtid,
                                       uint64_t gstride) {
    const uint32_t md = f.max_draws, lane = threadIdx.x & 31;
    if (gtid == 0) {
        f.status[kStRasterClaim] = 0u;
        f.status[kStBigClaim] = 0u;
        *reinterpret_cast<unsigned long long*>(f.status + kStBigPacked) = 0ull;
    }
    for (uint32_t v = 0; v < n_views; v++) {
        const ViewDev* vw = f.views + view_begin + v;
        if (vw->kind != kViewVisibility || !vw->lists) continue;
        const uint32_t* cnt = reinterpret_cast<const uint32_t*>(vw->draws);
        const uint32_t nop = min(cnt[0], md), nal = min(cnt[1], md);
        const lh_mat4& pv = vw->uniforms->combined_perspective_view;
        const uint64_t n = (uint64_t)nop + nal;
        // whole warps iterate together (the appends are warp collectives)
        for (uint64_t base = gtid - lane; base < n; base += gstride) {
            const uint64_t i = base + lane;
            bool keep = false, alpha = false;
            uint32_t slot = 0;
            if (i < n) {
                alpha = i >= nop;
                slot = alpha ? md + (uint32_t)(i - nop) : (uint32_t)i;
                const RasterDraw* rd = vw->rdraws + slot;
                // both loads issued together (one round trip)
                const uint32_t bits = __ldcg(&rd->bits);
                const float4 sp4 = __ldcg(reinterpret_cast<const float4*>(rd->sphere));
                if (!(bits & (kDrawOccluder | kDrawNoCentre))) {
                    const float sp[4] = {sp4.x, sp4.y, sp4.z, sp4.w};
                    keep = !vw->hiz || !hiz_occluded(vw, pv, sp);
                }
            }
#pragma unroll
            for (int cl = 0; cl < 2; cl++) {
                const bool mine = keep && (alpha == (cl == 1));
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, mine);
                if (!m) continue;
                const uint32_t leader = __ffs(m) - 1;
                uint32_t first = 0;
                if (lane == leader) first = atomicAdd(&vw->claim[cl ? kClaimSurvivorsAlpha : kClaimSurvivorsOpaque], __popc(m));
                first = __shfl_sync(0xFFFFFFFFu, first, leader);
                const uint32_t pos = first + __popc(m & ((1u << lane) - 1u));
                if (mine && pos < md) vw->lists[(size_t)(cl ? 2u : 1u) * md + pos] = slot;
            }
        }
    }
}

}  // namespace
}  // namespace lh
