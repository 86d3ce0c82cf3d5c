// Frame set-up, min/max depth reduction and the cascade fit as device
// phases (shared by the per-stage kernels and the persistent kernel).
//
// Reference passes: reset_buffers_a/b/c (src/shaders/compute/
// reset_buffers.glsl:9-57), read_depth (compute/read_depth.glsl:22-83),
// generate_shadow_matrices (compute/generate_shadow_matrices.glsl:15-110).
#pragma once

#include "lh_device.cuh"
#include "lh_internal.cuh"

namespace lh {
namespace {

// ---------------------------------------------------------------- frame set-up
// grid = (blocks, n_views): clears each view's target (visibility 0, shadow
// depth 1.0) with 16-byte stores; block (0, 0) also resets the per-view
// counters and the depth range (reset_buffers.glsl:9-29, util.glsl:61-70).
// Clear the target of view `view` with threads gtid of gstride; the thread
// with `reset_counters` also resets the per-view counters and depth range.
// Per-view counters and the depth range (one block).
__device__ void reset_view_counters(const FrameDev& f) {
    for (uint32_t v = threadIdx.x; v < f.n_views; v += blockDim.x) {
        *reinterpret_cast<unsigned long long*>(f.views[v].sector) = 0ull;
        *reinterpret_cast<unsigned long long*>(f.views[v].draws) = 0ull;
    }
    if (threadIdx.x == 0) {
        f.misc->min_depth = 0xFFFFFFFFu;
        f.misc->max_depth = 0u;
    }
}

__device__ void phase_clear_view(const FrameDev& f, uint32_t view, uint64_t tid, uint64_t stride, bool reset_counters) {
    const ViewDev* vw = f.views + view;
    const uint64_t npx = (uint64_t)vw->width * vw->height;
    if (vw->kind == kViewVisibility) {
        uint4* p = reinterpret_cast<uint4*>(vw->target);
        const uint64_t n = npx / 2;
        for (uint64_t i = tid; i < n; i += stride) p[i] = make_uint4(0, 0, 0, 0);
        if ((npx & 1) && tid == 0) reinterpret_cast<unsigned long long*>(vw->target)[npx - 1] = 0ull;
    } else {
        const uint32_t one = 0x3F800000u;
        uint4* p = reinterpret_cast<uint4*>(vw->target);
        const uint64_t n = npx / 4;
        for (uint64_t i = tid; i < n; i += stride) p[i] = make_uint4(one, one, one, one);
        for (uint64_t i = n * 4 + tid; i < npx; i += stride) reinterpret_cast<uint32_t*>(vw->target)[i] = one;
    }
    if (reset_counters) reset_view_counters(f);
}

// ---------------------------------------------------------------- cascade fit
// matrices.glsl:9-19
__device__ lh_mat4 look_at(f3 eye, f3 at, f3 up) {
    f3 fw = normalize(at - eye);
    f3 r = normalize(cross(fw, up));
    f3 u = cross(r, fw);
    lh_mat4 m;
    m.cols[0] = {r.x, u.x, -fw.x, 0.0f};
    m.cols[1] = {r.y, u.y, -fw.y, 0.0f};
    m.cols[2] = {r.z, u.z, -fw.z, 0.0f};
    m.cols[3] = {-dot(r, eye), -dot(u, eye), dot(fw, eye), 1.0f};
    return m;
}
// matrices.glsl:21-40
__device__ lh_mat4 orthographic(float left, float right, float bottom, float top, float n, float fr) {
    float rml = right - left, rpl = right + left, tmb = top - bottom, tpb = top + bottom, fmn = fr - n;
    lh_mat4 m;
    m.cols[0] = {2.0f / rml, 0.0f, 0.0f, 0.0f};
    m.cols[1] = {0.0f, -2.0f / tmb, 0.0f, 0.0f};
    m.cols[2] = {0.0f, 0.0f, -1.0f / fmn, 0.0f};
    m.cols[3] = {-(rpl / rml), -(tpb / tmb), -(n / fmn), 1.0f};
    return m;
}
__device__ lh_mat4 matmul(const lh_mat4& a, const lh_mat4& b) {
    lh_mat4 r;
    for (int c = 0; c < 4; c++) {
        f4 v = mul(a, f4{b.cols[c].x, b.cols[c].y, b.cols[c].z, b.cols[c].w});
        r.cols[c] = {v.x, v.y, v.z, v.w};
    }
    return r;
}

// generate_shadow_matrices.glsl:15-110 for cascade c.  pow(0.5, split) and
// pow(0.75, split) arrive precomputed (host, double, rounded to float).
__device__ void fit_cascade(const FrameDev& f, uint32_t c, uint32_t min_bits, uint32_t max_bits) {
    const Uniforms& u = *f.uniforms;
    MiscStorage& m = *f.misc;
    float min_depth = u2f(min_bits), max_depth = u2f(max_bits);
    float min_distance = NEAR_PLANE / max_depth;
    float max_distance = NEAR_PLANE / min_depth;
    float p05 = f.frame_consts[0], p075 = f.frame_consts[1];
    float splits[4] = {max_depth, NEAR_PLANE / (min_distance * (1.0f - p05) + max_distance * p05),
                       NEAR_PLANE / (min_distance * (1.0f - p075) + max_distance * p075), min_depth};
    float last = c > 0 ? splits[c - 1] : max_depth;
    float split = splits[c];
    f3 corners[8] = {{-1.0f, 1.0f, last},  {1.0f, 1.0f, last},  {1.0f, -1.0f, last},  {-1.0f, -1.0f, last},
                     {-1.0f, 1.0f, split}, {1.0f, 1.0f, split}, {1.0f, -1.0f, split}, {-1.0f, -1.0f, split}};
    for (int i = 0; i < 8; i++) {
        f4 ic = mul(u.inv_perspective_view, f4{corners[i].x, corners[i].y, corners[i].z, 1.0f});
        corners[i] = f3{ic.x / ic.w, ic.y / ic.w, ic.z / ic.w};
    }
    f3 center{0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 8; i++) center = center + corners[i];
    center = center / 8.0f;
    float radius = 0.0f;
    for (int i = 0; i < 8; i++) radius = gmax(radius, length(corners[i] - center));
    radius = ceilf(radius * 16.0f) / 16.0f;
    f3 eye = ld3(u.sun_dir) * u.shadow_cam_distance + center;
    lh_mat4 view = look_at(eye, center, f3{0.0f, 1.0f, 0.0f});
    lh_mat4 proj = orthographic(-radius, radius, -radius, radius, 0.0f, u.shadow_cam_distance * 2.0f);
    lh_mat4 mat = matmul(proj, view);
    lh_mat4 bias;
    bias.cols[0] = {0.5f, 0.0f, 0.0f, 0.0f};
    bias.cols[1] = {0.0f, 0.5f, 0.0f, 0.0f};
    bias.cols[2] = {0.0f, 0.0f, 1.0f, 0.0f};
    bias.cols[3] = {0.5f, 0.5f, 0.0f, 1.0f};
    m.shadow_matrices[c] = mat;
    m.uv_space_shadow_matrices[c] = matmul(bias, mat);
    m.shadow_view_matrices[c] = view;
    m.shadow_sphere_radii[c] = radius;
}

// Min over non-zero depth bits and max over all depth bits of the main view
// (read_depth.glsl:3-18,57-82: the 4x4 gathers with clamp-to-edge visit
// every texel), reduced per warp and merged with one atomic per warp.
__device__ void phase_depth_reduce(const FrameDev& f, uint64_t tid, uint64_t stride) {
    const uint64_t npx = (uint64_t)f.uniforms->window_size.x * f.uniforms->window_size.y;
    uint32_t mn = 0xFFFFFFFFu, mx = 0u;
    const uint4* p = reinterpret_cast<const uint4*>(f.visibility);
    const uint64_t n2 = npx / 2;
#pragma unroll 4
    for (uint64_t i = tid; i < n2; i += stride) {
        uint4 v = __ldcs(p + i);  // streaming: each pixel is read once
        uint32_t d0 = v.y, d1 = v.w;
        mx = max(mx, max(d0, d1));
        if (d0) mn = min(mn, d0);
        if (d1) mn = min(mn, d1);
    }
    if ((npx & 1) && tid == 0) {
        uint32_t d = (uint32_t)(reinterpret_cast<const unsigned long long*>(f.visibility)[npx - 1] >> 32);
        mx = max(mx, d);
        if (d) mn = min(mn, d);
    }
    mn = __reduce_min_sync(0xFFFFFFFFu, mn);
    mx = __reduce_max_sync(0xFFFFFFFFu, mx);
    // then across the block's warps: one pair of atomics per block
    __shared__ uint32_t s_mn[32], s_mx[32];
    const uint32_t warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_mn[warp] = mn;
        s_mx[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        mn = threadIdx.x < nwarps ? s_mn[threadIdx.x] : 0xFFFFFFFFu;
        mx = threadIdx.x < nwarps ? s_mx[threadIdx.x] : 0u;
        mn = __reduce_min_sync(0xFFFFFFFFu, mn);
        mx = __reduce_max_sync(0xFFFFFFFFu, mx);
        if (threadIdx.x == 0) {
            if (mn != 0xFFFFFFFFu) atomicMin(&f.misc->min_depth, mn);
            atomicMax(&f.misc->max_depth, mx);
        }
    }
}

// The 4 cascade fits, threads 0..3 of one block, after the reduction.
__device__ void phase_fit(const FrameDev& f) {
    __threadfence();
    const uint32_t min_bits = atomicOr(&f.misc->min_depth, 0u), max_bits = atomicOr(&f.misc->max_depth, 0u);
    if (threadIdx.x == 0 && min_bits == 0xFFFFFFFFu) atomicOr(&f.status[kStFlags], LH_FLAG_NO_DEPTH);
    if (threadIdx.x < 4) fit_cascade(f, threadIdx.x, min_bits, max_bits);
}

}  // namespace
}  // namespace lh
