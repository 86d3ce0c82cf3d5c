// Display transform (src/shaders/display_transform.comp:5-81): the
// scene-referred HDR image through a 48^3 LUT tonemap (tony_mc_mapface's
// encoding: stimulus / (stimulus + 1), LUT sampled trilinearly with clamp to
// edge at texel centres), the optional cascade overlay of debug_shadowmaps,
// and the sRGB transfer function, written as RGBA8.  The reference's LUT
// (external/tony-mc-mapface) is an empty submodule here, so callers pass
// their LUT or get a stand-in identity LUT (display = stimulus / (1 +
// stimulus) per channel).
#include "frame_phases.cuh"

namespace lh {
namespace {

constexpr int kLutDims = 48;

// Trilinear sample of a float4[48][48][48] LUT (x fastest) at normalised
// coordinates, clamp to edge.
__device__ __forceinline__ f3 lut_sample(const float4* lut, f3 uvw) {
    const float tx = uvw.x * (float)kLutDims - 0.5f, ty = uvw.y * (float)kLutDims - 0.5f,
                tz = uvw.z * (float)kLutDims - 0.5f;
    const float fx = floorf(tx), fy = floorf(ty), fz = floorf(tz);
    const float a = tx - fx, b = ty - fy, c = tz - fz;
    auto cl = [](int i) { return i < 0 ? 0 : (i > kLutDims - 1 ? kLutDims - 1 : i); };
    const int x0 = cl((int)fx), x1 = cl((int)fx + 1), y0 = cl((int)fy), y1 = cl((int)fy + 1), z0 = cl((int)fz),
              z1 = cl((int)fz + 1);
    auto t = [&](int x, int y, int z) {
        const float4 v = __ldg(lut + ((size_t)z * kLutDims + y) * kLutDims + x);
        return f3{v.x, v.y, v.z};
    };
    const f3 c00 = t(x0, y0, z0) * (1.0f - a) + t(x1, y0, z0) * a, c10 = t(x0, y1, z0) * (1.0f - a) + t(x1, y1, z0) * a;
    const f3 c01 = t(x0, y0, z1) * (1.0f - a) + t(x1, y0, z1) * a, c11 = t(x0, y1, z1) * (1.0f - a) + t(x1, y1, z1) * a;
    const f3 c0 = c00 * (1.0f - b) + c10 * b, c1 = c01 * (1.0f - b) + c11 * b;
    return c0 * (1.0f - c) + c1 * c;
}

// Bilinear sample (clamp to edge) of shadow layer `layer` at uv.
__device__ __forceinline__ float shadow_texel_bilinear(const float* maps, uint32_t S, uint32_t layer, float u, float v) {
    const float* m = maps + (size_t)layer * S * S;
    const float tu = u * (float)S - 0.5f, tv = v * (float)S - 0.5f;
    const float fu = floorf(tu), fv = floorf(tv);
    const float a = tu - fu, b = tv - fv;
    auto cl = [&](int i) { return i < 0 ? 0 : (i > (int)S - 1 ? (int)S - 1 : i); };
    const int i0 = cl((int)fu), i1 = cl((int)fu + 1), j0 = cl((int)fv), j1 = cl((int)fv + 1);
    const float t00 = __ldg(m + (size_t)j0 * S + i0), t10 = __ldg(m + (size_t)j0 * S + i1),
                t01 = __ldg(m + (size_t)j1 * S + i0), t11 = __ldg(m + (size_t)j1 * S + i1);
    return ((t00 * ((1.0f - a) * (1.0f - b)) + t10 * (a * (1.0f - b))) + t01 * ((1.0f - a) * b)) + t11 * (a * b);
}

__device__ __forceinline__ float srgb_oetf(float v) {
    return v <= 0.003130f ? v * 12.92f : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
}

__device__ __forceinline__ uint32_t unorm8(float v) {
    v = v > 0.0f ? v : 0.0f;
    v = v < 1.0f ? v : 1.0f;
    return (uint32_t)floorf(v * 255.0f + 0.5f);
}

// One thread per pixel (blocks of 32 x 8).
__global__ void __launch_bounds__(256) k_display_transform(FrameDev f, const float4* lut, uchar4* out) {
    pdl_enter();
    const Uniforms& u = *f.uniforms;
    const uint32_t W = u.window_size.x, H = u.window_size.y;
    const uint32_t x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= W || y >= H) return;
    const float4 hdr = load_hdr(f.hdr, f.hdr_half, (size_t)y * W + x);
    const f3 stimulus{hdr.x, hdr.y, hdr.z};
    // tony_mc_mapface (display_transform.comp:5-17)
    const f3 encoded{stimulus.x / (stimulus.x + 1.0f), stimulus.y / (stimulus.y + 1.0f),
                     stimulus.z / (stimulus.z + 1.0f)};
    const float scale = ((float)kLutDims - 1.0f) / (float)kLutDims, bias = 0.5f / (float)kLutDims;
    f3 v = lut_sample(lut, f3{encoded.x * scale + bias, encoded.y * scale + bias, encoded.z * scale + bias});
    if (u.debug_shadowmaps) {
        // display_transform.comp:51-75
        const float uvx = ((float)x + 0.5f) / (float)W, uvy = ((float)y + 0.5f) / (float)H;
        const float pct = 0.5f;
        if (uvx < pct && uvy < pct) {
            const float sx = uvx * 2.0f / pct, sy = uvy * 2.0f / pct;
            const uint32_t cascade = (sy > 1.0f ? 2u : 0u) + (sx > 1.0f ? 1u : 0u);
            const float d = shadow_texel_bilinear(f.shadow_maps, f.shadow_size, cascade, sx - floorf(sx), sy - floorf(sy));
            const float g = (d - 0.5f) * 100.0f + 0.5f;
            v = f3{g, g, g};
        }
    }
    out[(size_t)y * W + x] = make_uchar4((unsigned char)unorm8(srgb_oetf(v.x)), (unsigned char)unorm8(srgb_oetf(v.y)),
                                         (unsigned char)unorm8(srgb_oetf(v.z)), 255);
}

}  // namespace

cudaError_t launch_display_transform(const FrameDev& f, uint32_t width, uint32_t height, const float4* lut, uchar4* out,
                                     cudaStream_t s) {
    dim3 grid((width + 31) / 32, (height + 7) / 8);
    return launch_pdl(k_display_transform, grid, dim3(32, 8), s, f, lut, out);
}

}  // namespace lh
