// Frame set-up, min/max depth reduction fused with the cascade fit, and the
// full-screen lighting resolve.
//
// Reference passes: reset_buffers_a/b/c (src/shaders/compute/
// reset_buffers.glsl:9-57), read_depth (compute/read_depth.glsl:22-83),
// generate_shadow_matrices (compute/generate_shadow_matrices.glsl:15-110) and
// render_geometry (src/shaders/render_geometry.comp:70-266).
#include <algorithm>
#include <cstring>

#include "exact_div.cuh"
#include "frame_phases.cuh"
#include "tma.cuh"

namespace lh {
namespace {

// ---------------------------------------------------------------- resolve
struct Tex4 { float r, g, b, a; };

// Bilinear filtering of level 0 with repeat addressing, over the texture's
// linear float4 copy.
// A 1 x 1 texture (the scenes' constant materials) returns its texel: the
// bilinear blend of four copies of one value is that value up to rounding.
__device__ Tex4 sample_repeat(const FrameDev& f, uint32_t index, f2 uv) {
    if (index >= f.n_textures) return {0.0f, 0.0f, 0.0f, 0.0f};
    const lh_texture t = f.textures[index];
    const float4* tex = f.tex_linear[index];
    if (t.width == 1 && t.height == 1) {
        const float4 p = __ldg(tex);
        return Tex4{p.x, p.y, p.z, p.w};
    }
    float u = uv.x * (float)t.width - 0.5f, v = uv.y * (float)t.height - 0.5f;
    if (!(fabsf(u) < 1e9f)) u = 0.0f;
    if (!(fabsf(v) < 1e9f)) v = 0.0f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    const int32_t i0 = (int32_t)fu, j0 = (int32_t)fv;
    const int32_t W = (int32_t)t.width, H = (int32_t)t.height;
    // i0 + 1 wraps to the texel after i0's (or 0 past the last)
    const int32_t ia = wrap_texel(i0, W), ib = ia + 1 == W ? 0 : ia + 1;
    const int32_t ja = wrap_texel(j0, H), jb = ja + 1 == H ? 0 : ja + 1;
    const float4* row_a = tex + (size_t)ja * W;
    const float4* row_b = tex + (size_t)jb * W;
    auto texel = [&](const float4* row, int32_t i) {
        const float4 p = __ldg(row + i);
        return Tex4{p.x, p.y, p.z, p.w};
    };
    Tex4 t00 = texel(row_a, ia), t10 = texel(row_a, ib), t01 = texel(row_b, ia), t11 = texel(row_b, ib);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    Tex4 r;
    r.r = ((t00.r * w00 + t10.r * w10) + t01.r * w01) + t11.r * w11;
    r.g = ((t00.g * w00 + t10.g * w10) + t01.g * w01) + t11.g * w11;
    r.b = ((t00.b * w00 + t10.b * w10) + t01.b * w01) + t11.b * w11;
    r.a = ((t00.a * w00 + t10.a * w10) + t01.a * w01) + t11.a * w11;
    return r;
}

// Comparison sampling (compare op LESS, linear, clamp to edge) of layer
// clamp(round(layer), 0, 3).
__device__ float sample_shadow(const FrameDev& f, f2 uv, float layer_f, float ref) {
    int layer = __float2int_rn(layer_f);
    layer = min(max(layer, 0), 3);
    const uint32_t S = f.shadow_size;
    const float* map = f.shadow_maps + (size_t)layer * S * S;
    float u = uv.x * (float)S - 0.5f, v = uv.y * (float)S - 0.5f;
    if (!(fabsf(u) < 1e9f)) u = 0.0f;
    if (!(fabsf(v) < 1e9f)) v = 0.0f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    const int32_t i0 = (int32_t)fu, j0 = (int32_t)fv;
    auto cl = [&](int32_t i) { return i < 0 ? 0 : (i > (int32_t)S - 1 ? (int32_t)S - 1 : i); };
    auto cmp = [&](int32_t i, int32_t j) { return ref < __ldg(map + (size_t)cl(j) * S + cl(i)) ? 1.0f : 0.0f; };
    float c00 = cmp(i0, j0), c10 = cmp(i0 + 1, j0), c01 = cmp(i0, j0 + 1), c11 = cmp(i0 + 1, j0 + 1);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return ((c00 * w00 + c10 * w10) + c01 * w01) + c11 * w11;
}

// The 9-tap PCF of render_geometry.comp:200-214 at shadow coordinate
// (sx, sy), reference depth `ref`: the sum of sample_shadow over the taps
// at offsets (ox, oy) / 1024.  When the taps' texel columns and rows are
// consecutive (a 1024-texel cascade: the offsets are one texel apart) the
// 4 x 4 texels they share are compared once -- 16 loads instead of 36 -- and
// the sum is taken in separable form: tap (ox, oy) weighs its 2 x 2 texels by
// (1 - a_ox, a_ox) x (1 - b_oy, b_oy), so texel (i, j) of the window carries
// CX(i) * CY(j) with CX = (1 - a_0, a_0 + 1 - a_1, a_1 + 1 - a_2, a_2) and CY
// alike: the same compare results, the same weights, summed in another
// order (float rounding only).  Otherwise tap by tap.
__device__ float pcf9(const FrameDev& f, float sx, float sy, float layer_f, float ref) {
    const uint32_t S = f.shadow_size;
    float ax[3], ay[3];
    int32_t ix[3], iy[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        // (the middle tap's offset is +0: sx + 0 only turns -0 into +0, which
        // gives the same u)
        float u = (k == 1 ? sx : sx + (float)(k - 1) / 1024.0f) * (float)S - 0.5f;
        float v = (k == 1 ? sy : sy + (float)(k - 1) / 1024.0f) * (float)S - 0.5f;
        if (!(fabsf(u) < 1e9f)) u = 0.0f;
        if (!(fabsf(v) < 1e9f)) v = 0.0f;
        const float fu = floorf(u), fv = floorf(v);
        ax[k] = u - fu;
        ay[k] = v - fv;
        ix[k] = (int32_t)fu;
        iy[k] = (int32_t)fv;
    }
    if (ix[1] == ix[0] + 1 && ix[2] == ix[1] + 1 && iy[1] == iy[0] + 1 && iy[2] == iy[1] + 1) {
        int layer = __float2int_rn(layer_f);
        layer = min(max(layer, 0), 3);
        const float* map = f.shadow_maps + (size_t)layer * S * S;
        auto cl = [&](int32_t i) { return i < 0 ? 0 : (i > (int32_t)S - 1 ? (int32_t)S - 1 : i); };
        const float cx[4] = {1.0f - ax[0], ax[0] + (1.0f - ax[1]), ax[1] + (1.0f - ax[2]), ax[2]};
        const float cy[4] = {1.0f - ay[0], ay[0] + (1.0f - ay[1]), ay[1] + (1.0f - ay[2]), ay[2]};
        // each row's passing texels weighted by their column weights as they
        // are compared (a texel that fails adds +0: with no texel passing the
        // sum is exactly +0)
        float sum = 0.0f;
        if (ix[0] >= 0 && iy[0] >= 0 && ix[0] <= (int32_t)S - 4 && iy[0] <= (int32_t)S - 4) {
            // the window inside the map: no clamping, four consecutive texels a row
            const float* row = map + (size_t)iy[0] * S + ix[0];
#pragma unroll
            for (int r = 0; r < 4; r++, row += S) {
                const float w0 = ref < __ldg(row) ? cx[0] : 0.0f, w1 = ref < __ldg(row + 1) ? cx[1] : 0.0f;
                const float w2 = ref < __ldg(row + 2) ? cx[2] : 0.0f, w3 = ref < __ldg(row + 3) ? cx[3] : 0.0f;
                sum = __fmaf_rn((w0 + w1) + (w2 + w3), cy[r], sum);
            }
            return sum;
        }
        int32_t col[4];
#pragma unroll
        for (int c = 0; c < 4; c++) col[c] = cl(ix[0] + c);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const float* row = map + (size_t)cl(iy[0] + r) * S;
            const float w0 = ref < __ldg(row + col[0]) ? cx[0] : 0.0f, w1 = ref < __ldg(row + col[1]) ? cx[1] : 0.0f;
            const float w2 = ref < __ldg(row + col[2]) ? cx[2] : 0.0f, w3 = ref < __ldg(row + col[3]) ? cx[3] : 0.0f;
            sum = __fmaf_rn((w0 + w1) + (w2 + w3), cy[r], sum);
        }
        return sum;
    }
    float sum = 0.0f;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = -1; oy <= 1; oy++) {
            f2 off{(float)ox / 1024.0f, (float)oy / 1024.0f};
            sum += sample_shadow(f, f2{sx + off.x, sy + off.y}, layer_f, ref);
        }
    return sum;
}

constexpr float kPi = 3.14159265358979323846f;

// pbr.glsl:3-96
// The BRDF feeds no discrete decision, so it runs on approximate division,
// reciprocal square root and multiplied-out integer powers (a few ulp; the
// radiance is checked at 2^-10).  Everything that selects something -- the
// barycentrics and world position (cascade, PCF taps, compare results) and
// the view vector (face flip) -- stays in the oracle's IEEE arithmetic.
__device__ __forceinline__ float pow5f(float x) {
    const float x2 = x * x;
    return x2 * x2 * x;
}
__device__ __forceinline__ f3 fast_normalize(f3 v) { return v * rsqrtf(dot(v, v)); }
__device__ __forceinline__ float F_Schlick1(float u, float f0, float f90) { return f0 + (f90 - f0) * pow5f(1.0f - u); }
__device__ __forceinline__ float Fd_Burley(float NoV, float NoL, float LoH, float rough) {
    float f90 = 0.5f + 2.0f * rough * LoH * LoH;
    float light = F_Schlick1(NoL, 1.0f, f90);
    float view = F_Schlick1(NoV, 1.0f, f90);
    return light * view * (1.0f / kPi);
}
__device__ __forceinline__ float D_GGX(float NoH, float a) {
    float a2 = a * a;
    float fq = (NoH * a2 - NoH) * NoH + 1.0f;
    return __fdividef(a2, kPi * fq * fq);
}
__device__ __forceinline__ float V_SmithGGXCorrelated(float NoV, float NoL, float a) {
    float a2 = a * a;
    float GGXL = NoV * sqrtf((-NoL * a2 + NoL) * NoL + a2);
    float GGXV = NoL * sqrtf((-NoV * a2 + NoV) * NoV + a2);
    return __fdividef(0.5f, GGXV + GGXL);
}
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ f3 BRDF(f3 v, f3 l, f3 n, float pr, float metallic, f3 base, bool thin) {
    f3 h = fast_normalize(v + l);
    f3 diffuse = base * (1.0f - metallic);
    float refl = (1.5f - 1.0f) / (1.5f + 1.0f);
    refl = refl * refl;
    f3 f0 = f3{refl, refl, refl} * (1.0f - metallic) + base * metallic;
    float NoV = clampf(dot(n, v), 1e-5f, 1.0f);
    float NoL = clampf(dot(n, l), 0.0f, 1.0f);
    float NoH = clampf(dot(n, h), 0.0f, 1.0f);
    float LoH = clampf(dot(l, h), 0.0f, 1.0f);
    float rough = pr * pr;
    float D = D_GGX(NoH, rough);
    float p = pow5f(1.0f - LoH);
    f3 F{f0.x + (1.0f - f0.x) * p, f0.y + (1.0f - f0.y) * p, f0.z + (1.0f - f0.z) * p};
    float V = V_SmithGGXCorrelated(NoV, NoL, rough);
    f3 Fr = F * (D * V);
    f3 Fd = diffuse * Fd_Burley(NoV, NoL, LoH, rough);
    f3 irr = (Fd + Fr) * NoL;
    irr = f3{gmax(irr.x, 0.0f), gmax(irr.y, 0.0f), gmax(irr.z, 0.0f)};
    if (thin) {
        float rNoV = clampf(dot(-n, v), 1e-5f, 1.0f);
        float rNoL = clampf(dot(-n, l), 0.0f, 1.0f);
        irr = irr + diffuse * Fd_Burley(rNoV, rNoL, LoH, rough) * rNoL;
    }
    return {isnan(irr.x) ? 0.0f : irr.x, isnan(irr.y) ? 0.0f : irr.y, isnan(irr.z) ? 0.0f : irr.z};
}

struct Bary { f3 lambda, ddx, ddy; };

// vbuffer.glsl:11-63.  kDeriv: also the screen derivatives of lambda, which
// only the normal-map path reads (computed there, not for every pixel).
// A clip-space vertex as the barycentrics read it: 1 / w and the projected
// x, y (a vertex's own terms, so the resolve's vertex stage computes them
// once per vertex for every pixel of the triangle).
struct ProjVertex { float inv_w; f2 n; };
__device__ __forceinline__ ProjVertex project_vertex(f4 p) {
    const float iw = 1.0f / p.w;
    return {iw, f2{p.x * iw, p.y * iw}};
}
template <bool kDeriv>
__device__ Bary calc_full_bary(ProjVertex v0, ProjVertex v1, ProjVertex v2, f2 ndc, f2 win) {
    Bary r;
    f3 invW{v0.inv_w, v1.inv_w, v2.inv_w};
    const f2 n0 = v0.n, n1 = v1.n, n2 = v2.n;
    f2 ca{n2.x - n1.x, n2.y - n1.y}, cb{n0.x - n1.x, n0.y - n1.y};
    float invDet = 1.0f / (ca.x * cb.y - cb.x * ca.y);
    r.ddx = f3{n1.y - n2.y, n2.y - n0.y, n0.y - n1.y} * invDet * invW;
    r.ddy = f3{n2.x - n1.x, n0.x - n2.x, n1.x - n0.x} * invDet * invW;
    float ddxSum = dot(r.ddx, f3{1.0f, 1.0f, 1.0f});
    float ddySum = dot(r.ddy, f3{1.0f, 1.0f, 1.0f});
    f2 dv{ndc.x - n0.x, ndc.y - n0.y};
    float interpInvW = (invW.x + dv.x * ddxSum) + dv.y * ddySum;
    float interpW = 1.0f / interpInvW;
    r.lambda.x = interpW * ((invW.x + dv.x * r.ddx.x) + dv.y * r.ddy.x);
    r.lambda.y = interpW * ((0.0f + dv.x * r.ddx.y) + dv.y * r.ddy.y);
    r.lambda.z = interpW * ((0.0f + dv.x * r.ddx.z) + dv.y * r.ddy.z);
    if (!kDeriv) return r;
    r.ddx = r.ddx * (2.0f / win.x);
    r.ddy = r.ddy * (2.0f / win.y);
    ddxSum *= 2.0f / win.x;
    ddySum *= 2.0f / win.y;
    r.ddy = r.ddy * -1.0f;
    ddySum *= -1.0f;
    float interpW_ddx = 1.0f / (interpInvW + ddxSum);
    float interpW_ddy = 1.0f / (interpInvW + ddySum);
    r.ddx = (r.lambda * interpInvW + r.ddx) * interpW_ddx - r.lambda;
    r.ddy = (r.lambda * interpInvW + r.ddy) * interpW_ddy - r.lambda;
    return r;
}
__device__ __forceinline__ f3 interp_deriv(const Bary& b, float v0, float v1, float v2) {
    f3 m{v0, v1, v2};
    return {dot(m, b.lambda), dot(m, b.ddx), dot(m, b.ddy)};
}

// DEBUG_COLOURS (shaders/common/debug.glsl:1-11) and temperature()
// (debug.glsl:15-37) for the debug views.
__constant__ float c_debug_colours[10][3] = {
    {0.0f / 255.0f, 2.0f / 255.0f, 91.0f / 255.0f},     {0.0f / 255.0f, 108.0f / 255.0f, 251.0f / 255.0f},
    {0.0f / 255.0f, 221.0f / 255.0f, 221.0f / 255.0f},  {51.0f / 255.0f, 221.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 252.0f / 255.0f, 0.0f / 255.0f},  {255.0f / 255.0f, 180.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 104.0f / 255.0f, 0.0f / 255.0f},  {226.0f / 255.0f, 22.0f / 255.0f, 0.0f / 255.0f},
    {191.0f / 255.0f, 0.0f / 255.0f, 83.0f / 255.0f},   {145.0f / 255.0f, 0.0f / 255.0f, 65.0f / 255.0f}};
__device__ __forceinline__ f3 debug_colour(uint32_t i) {
    return {c_debug_colours[i][0], c_debug_colours[i][1], c_debug_colours[i][2]};
}
__device__ __forceinline__ float smoothstep_(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}
__device__ f3 temperature(float t) {
    const float s = t * 10.0f;
    const int cur = (int)s <= 9 ? (int)s : 9;
    const int prv = cur >= 1 ? cur - 1 : 0;
    const int nxt = cur < 9 ? cur + 1 : 9;
    const float blur = 0.8f;
    const float wc = smoothstep_((float)cur - blur, (float)cur + blur, s) *
                     (1.0f - smoothstep_((float)(cur + 1) - blur, (float)(cur + 1) + blur, s));
    const float wp = 1.0f - smoothstep_((float)cur - blur, (float)cur + blur, s);
    const float wn = smoothstep_((float)(cur + 1) - blur, (float)(cur + 1) + blur, s);
    const f3 r = debug_colour(cur) * wc + debug_colour(prv) * wp + debug_colour(nxt) * wn;
    return {clampf(r.x, 0.0f, 1.0f), clampf(r.y, 0.0f, 1.0f), clampf(r.z, 0.0f, 1.0f)};
}

// The debug views (render_geometry.comp:268-308) that replace the lit
// colour with material / index / normal colours; not inlined, so the lit
// path's registers do not carry them.  They do not depend on the lighting,
// which the kernel then skips.
__device__ __noinline__ f3 debug_view(int32_t mode, f3 base, uint32_t cascade, uint32_t tri, uint32_t meshlet_index,
                                      f3 normal) {
    switch (mode) {
        case 1: return base * debug_colour(cascade);        // UNIFORMS_DEBUG_CASCADES
        case 2: return debug_colour(tri % 10);              // UNIFORMS_DEBUG_TRIANGLE_INDEX
        case 3: return debug_colour(meshlet_index % 10);    // UNIFORMS_DEBUG_INSTANCE_INDEX
        default: return normal * 0.5f + f3{0.5f, 0.5f, 0.5f};  // UNIFORMS_DEBUG_NORMALS
    }
}

// UNIFORMS_DEBUG_SHADER_CLOCK: the pixel's shading time as a heat map.
__device__ __noinline__ f3 clock_view(long long start_time) {
    const float dt = (float)(clock64() - start_time) / 65000.0f;
    return temperature(dt < 0.0f ? 0.0f : (dt > 1.0f ? 1.0f : dt));
}

// render_geometry.comp:70-308 for pixel (x, y) of the main view, whose
// visibility word is `vis`.
// Normal mapping (render_geometry.comp:25-38, 225-232): the cotangent frame
// from the screen derivatives of the world position and uv.  Not inlined:
// the scenes' materials rarely carry normal maps.
__device__ __noinline__ f3 apply_normal_map(const FrameDev& f, uint32_t tex, f2 uv, const lh_mat4& PV, f3 pa, f3 pb,
                                            f3 pc, f3 us, f3 vs, f2 ndc, f2 win, f3 normal) {
    Tex4 nt = sample_repeat(f, tex, uv);
    f3 mn{nt.r * 255.0f / 127.0f - 128.0f / 127.0f, nt.g * 255.0f / 127.0f - 128.0f / 127.0f,
          nt.b * 255.0f / 127.0f - 128.0f / 127.0f};
    // screen derivatives of the world position and uv (the same barycentrics
    // again, with their derivatives)
    const Bary bd = calc_full_bary<true>(project_vertex(mul(PV, f4{pa.x, pa.y, pa.z, 1.0f})),
                                         project_vertex(mul(PV, f4{pb.x, pb.y, pb.z, 1.0f})),
                                         project_vertex(mul(PV, f4{pc.x, pc.y, pc.z, 1.0f})), ndc, win);
    const f3 wx = interp_deriv(bd, pa.x, pb.x, pc.x), wy = interp_deriv(bd, pa.y, pb.y, pc.y),
             wz = interp_deriv(bd, pa.z, pb.z, pc.z);
    const f3 wdx{wx.y, wy.y, wz.y}, wdy{wx.z, wy.z, wz.z};
    const f3 uvx = interp_deriv(bd, us.x, us.y, us.z), uvy = interp_deriv(bd, vs.x, vs.y, vs.z);
    const f2 uvdx{uvx.y, uvy.y}, uvdy{uvx.z, uvy.z};
    f3 dpy = cross(wdy, normal), dpx = cross(normal, wdx);
    f3 t = dpy * uvdx.x + dpx * uvdy.x;
    f3 b = dpy * uvdx.y + dpx * uvdy.y;
    float invmax = 1.0f / sqrtf(gmax(dot(t, t), dot(b, b)));
    f3 tt = t * invmax, bb = b * invmax;
    return normalize(f3{(tt.x * mn.x + bb.x * mn.y) + normal.x * mn.z, (tt.y * mn.x + bb.y * mn.y) + normal.y * mn.z,
                        (tt.z * mn.x + bb.z * mn.y) + normal.z * mn.z});
}

// Vertex k of triangle `packed` (tri << 24 | draw slot) of the main view as
// the lighting reads it -- world position, clip position (PV times it)
// projected, normalised raw normal, uv times the texture scale -- in the
// arithmetic and order the lighting has always used.
__device__ __forceinline__ void load_vertex(const FrameDev& f, uint32_t packed, uint32_t k, f3& p, ProjVertex& c,
                                            f3& n, float& us, float& vs) {
    const uint32_t slot = packed & ((1u << 24) - 1u), tri = packed >> 24;
    const RasterDraw rd = f.views[0].rdraws[slot];
    const Instance* inst = f.instances + rd.instance;
    const MeshInfo* mip = mesh_info_of(inst);
    const uint32_t flags = rd.bits >> 16;
    const uint32_t vi = __ldg(reinterpret_cast<const uint8_t*>(rd.micro) + tri * 3 + k);
    const uint32_t idx = (flags & MESH_INFO_FLAGS_32_BIT_INDICES)
                             ? __ldg(reinterpret_cast<const uint32_t*>(rd.indices) + vi)
                             : __ldg(reinterpret_cast<const uint16_t*>(rd.indices) + vi);
    p = world_pos(inst->transform, load_position(rd.positions, flags, idx));
    c = project_vertex(mul(f.uniforms->combined_perspective_view, f4{p.x, p.y, p.z, 1.0f}));
    n = fast_normalize(load_normal_raw(__ldg(&mip->normals), flags, idx));
    const f2 uv = load_uv_raw(__ldg(&mip->uvs), flags, idx);
    us = uv.x * __ldg(&mip->texture_scale.x);
    vs = uv.y * __ldg(&mip->texture_scale.y);
}

constexpr uint32_t kShareTris = 10;  // distinct triangles a warp row shares vertex work for

// The vertex stage of a warp's 32 pixels (called by all lanes).  Neighbouring
// pixels mostly show one triangle (1.26 distinct triangles per 32-pixel row
// on average in the large workload), so the distinct triangles' vertices are
// computed once, one vertex per lane -- lanes 3q, 3q + 1, 3q + 2 for the q-th
// triangle to compute -- into the warp's shared-memory slots (3 float4 a
// vertex: p.xyz n.x | 1/w, projected x y | n.yz us vs), at a third of the
// vertex work of every pixel computing its own three.  The slots the warp's
// previous row segment used (`prev`, one bit a slot; s_keys holds each
// slot's triangle) are looked up first: a triangle that continues from the
// previous 32 pixels of the row keeps its vertices, and a segment whose
// triangles all continue computes none.  Returns the pixel's first vertex
// slot, or -1 when the row holds more than kShareTris distinct triangles
// (each pixel then computes its own at use; the slots stay as they were).
__device__ __forceinline__ int32_t share_vertices(const FrameDev& f, bool covered, uint32_t packed, uint32_t* s_keys,
                                                  float4* s_vert, uint32_t& prev) {
    const uint32_t lane = threadIdx.x;
    const uint32_t key = covered ? packed : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t leader = __ffs(peers) - 1;
    const bool lead = covered && lane == leader;
    const uint32_t leaders = __ballot_sync(0xFFFFFFFFu, lead);
    if (__popc(leaders) > kShareTris) return -1;
    int32_t slot = -1;
    for (uint32_t m = prev; m; m &= m - 1) {
        const uint32_t i = __ffs(m) - 1;
        if (s_keys[i] == key) slot = (int32_t)i;
    }
    const bool miss = lead && slot < 0;
    const uint32_t hits = __reduce_or_sync(0xFFFFFFFFu, lead && slot >= 0 ? 1u << slot : 0u);
    const uint32_t misses = __ballot_sync(0xFFFFFFFFu, miss);
    uint32_t used = hits;
    if (misses) {
        // the new triangles take slots that hold none of this segment's
        const uint32_t free = ~hits & ((1u << kShareTris) - 1u);
        if (miss) slot = (int32_t)__fns(free, 0, __popc(misses & ((1u << lane) - 1u)) + 1);
        used |= __reduce_or_sync(0xFFFFFFFFu, miss ? 1u << slot : 0u);
        __syncwarp();  // every lane's lookup has read s_keys, every pixel of the last segment its slots
        if (miss) s_keys[slot] = key;
        const uint32_t n_new = __popc(misses), q = lane / 3;
        const uint32_t src = q < n_new ? __fns(misses, 0, q + 1) : lane;
        const uint32_t qkey = __shfl_sync(0xFFFFFFFFu, key, src);
        const int32_t qslot = __shfl_sync(0xFFFFFFFFu, slot, src);
        if (q < n_new) {
            f3 p, nv;
            ProjVertex c;
            float us, vs;
            const uint32_t k = lane - 3 * q, v = 3 * (uint32_t)qslot + k;
            load_vertex(f, qkey, k, p, c, nv, us, vs);
            s_vert[3 * v] = make_float4(p.x, p.y, p.z, nv.x);
            s_vert[3 * v + 1] = make_float4(c.inv_w, c.n.x, c.n.y, 0.0f);
            s_vert[3 * v + 2] = make_float4(nv.y, nv.z, us, vs);
        }
        __syncwarp();
    }
    prev = used;
    slot = __shfl_sync(0xFFFFFFFFu, slot, leader);
    return covered ? 3 * slot : 0;
}

// Vertex k of the pixel's triangle: from the warp's slots, or computed.
__device__ __forceinline__ void pixel_vertex(const FrameDev& f, const float4* s_vert, int32_t base, uint32_t packed,
                                             uint32_t k, f3& p, ProjVertex& c, f3& n, float& us, float& vs) {
    if (base < 0) {
        load_vertex(f, packed, k, p, c, n, us, vs);
        return;
    }
    const float4 a = s_vert[3 * (base + k)], b = s_vert[3 * (base + k) + 1], d = s_vert[3 * (base + k) + 2];
    p = f3{a.x, a.y, a.z};
    c = ProjVertex{b.x, f2{b.y, b.z}};
    n = f3{a.w, d.x, d.y};
    us = d.z;
    vs = d.w;
}

// `clock_slot`: the thread's shared-memory word for the clock view's start
// time (kept out of registers).  Called by all lanes of the warp (the vertex
// stage is a warp collective); `in_view` false for lanes past the image.
// `s_uvs`: the block's shared copy of the 4 cascades' uv-space matrices;
// `rcp_w`: 1 / window width; `ndc_y`: the row's y / H * 2 - 1.
__device__ __forceinline__ void resolve_pixel(const FrameDev& f, uint32_t x, uint32_t y, unsigned long long vis,
                                              bool in_view, long long* clock_slot, uint32_t* s_keys, float4* s_vert,
                                              uint32_t& prev, const lh_mat4* s_uvs, float rcp_w, float ndc_y) {
    const Uniforms& u = *f.uniforms;
    if (in_view && u.debug == 4) *clock_slot = clock64();
    const int32_t vbase =
        share_vertices(f, in_view && u2f((uint32_t)(vis >> 32)) != 0.0f, (uint32_t)vis, s_keys, s_vert, prev);
    if (!in_view) return;
    const uint32_t W = u.window_size.x, H = u.window_size.y;
    // x / W * 2 - 1 with the quotient from the reciprocal (the same bits)
    const float qx = W <= (uint32_t)kExactDivMaxCount ? div_by_count((float)x, (float)W, rcp_w) : (float)x / (float)W;
    const f2 ndc{qx * 2.0f - 1.0f, ndc_y};
    const size_t pix = (size_t)y * W + x;
    if (u2f((uint32_t)(vis >> 32)) == 0.0f) {
        f4 un = mul(u.perspective_inverse, f4{ndc.x, ndc.y, 0.0f, 1.0f});
        f3 lr = normalize(f3{un.x, un.y, un.z});
        f4 r4 = mul(u.view_inverse, f4{lr.x, lr.y, lr.z, 0.0f});
        // procedural sky in place of the missing cubemap asset
        f3 s = f3{0.25f + 0.10f * r4.y, 0.35f + 0.15f * r4.y, 0.55f + 0.25f * r4.y} * powf(2.0f, 3.0f);
        store_hdr(f.hdr, f.hdr_half, pix, s.x, s.y, s.z);
        return;
    }
    const uint32_t packed = (uint32_t)vis;
    const uint32_t slot = packed & ((1u << 24) - 1u), tri = packed >> 24;
    // the slot's draw record (written by the meshlet cull): instance and
    // MeshInfo flags; the vertices came from the warp's vertex stage
    const RasterDraw rd = f.views[0].rdraws[slot];
    const Instance* inst = f.instances + rd.instance;
    const MeshInfoResolve mi = load_mesh_info_resolve(mesh_info_of(inst));
    const uint32_t flags = rd.bits >> 16;
    f3 pa, pb, pc, na, nb, nc;
    ProjVertex ca, cb, cc;
    f3 us, vs;
    pixel_vertex(f, s_vert, vbase, packed, 0, pa, ca, na, us.x, vs.x);
    pixel_vertex(f, s_vert, vbase, packed, 1, pb, cb, nb, us.y, vs.y);
    pixel_vertex(f, s_vert, vbase, packed, 2, pc, cc, nc, us.z, vs.z);
    const lh_mat4& PV = u.combined_perspective_view;
    const Bary bary = calc_full_bary<false>(ca, cb, cc, ndc, f2{(float)W, (float)H});
    const f3 world{dot(f3{pa.x, pb.x, pc.x}, bary.lambda), dot(f3{pa.y, pb.y, pc.y}, bary.lambda),
                   dot(f3{pa.z, pb.z, pc.z}, bary.lambda)};
    f2 uv{dot(us, bary.lambda) + mi.texture_offset.x, dot(vs, bary.lambda) + mi.texture_offset.y};
    f3 view_vector = normalize(ld3(u.camera_pos) - world);
    f3 normal{interp_deriv(bary, na.x, nb.x, nc.x).x, interp_deriv(bary, na.y, nb.y, nc.y).x,
              interp_deriv(bary, na.z, nb.z, nc.z).x};
    normal = fast_normalize(mul3(inst->normal_transform, normal));
    f3 gn = cross(pb - pa, pc - pa);
    if (dot(gn, view_vector) < 0.0f) normal = -normal;
    // materials first (they need the geometry the shadow code below does not,
    // so its registers free up early; the order changes no result)
    Tex4 bc = sample_repeat(f, mi.base_tex, uv);
    f3 base{bc.r * mi.base_color_factor.x, bc.g * mi.base_color_factor.y, bc.b * mi.base_color_factor.z};
    Tex4 mr = sample_repeat(f, mi.mr_tex, uv);
    float roughness = mr.g, metallic = mr.b;
    if (mi.normal_tex != UNUSED_TEXTURE_INDEX)
        normal = apply_normal_map(f, mi.normal_tex, uv, PV, pa, pb, pc, us, vs, ndc, f2{(float)W, (float)H}, normal);
    // the first cascade whose uv square holds the point (x and y of each
    // tried cascade, then z and w of the one taken -- the last tried when none
    // holds it -- in mul's operation order: the same values as the full
    // product per cascade)
    uint32_t ci;
    const f4 wp{world.x, world.y, world.z, 1.0f};
    f4 sc{0.0f, 0.0f, 0.0f, 0.0f};
    for (ci = 0; ci < 4; ci++) {
        const lh_vec4 &c0 = s_uvs[ci].cols[0], &c1 = s_uvs[ci].cols[1], &c2 = s_uvs[ci].cols[2],
                      &c3 = s_uvs[ci].cols[3];
        sc.x = ((c0.x * wp.x + c1.x * wp.y) + c2.x * wp.z) + c3.x * wp.w;
        sc.y = ((c0.y * wp.x + c1.y * wp.y) + c2.y * wp.z) + c3.y * wp.w;
        float ox = sc.x - 0.5f, oy = sc.y - 0.5f;
        if (fabsf(ox) < 0.5f && fabsf(oy) < 0.5f) break;
    }
    {
        const lh_mat4& m = s_uvs[ci < 4 ? ci : 3];
        sc.z = ((m.cols[0].z * wp.x + m.cols[1].z * wp.y) + m.cols[2].z * wp.z) + m.cols[3].z * wp.w;
        sc.w = ((m.cols[0].w * wp.x + m.cols[1].w * wp.y) + m.cols[2].w * wp.z) + m.cols[3].w * wp.w;
    }
    const bool alpha = (flags & MESH_INFO_FLAGS_ALPHA_CLIP) != 0;
    const float bias = alpha ? 0.000002f : 0.0f;
    // the cascade matrices are affine (w = 1 exactly for a finite point),
    // and x / 1 = x: the perspective divide only runs when it can change a bit
    if (sc.w != 1.0f) sc = f4{sc.x / sc.w, sc.y / sc.w, sc.z / sc.w, sc.w / sc.w};
    float shadow_sum = pcf9(f, sc.x, sc.y, (float)ci, sc.z - bias);
    shadow_sum = div_by_count(shadow_sum, 9.0f, 1.0f / 9.0f);  // shadow_sum / 9, the same bits
    if (sc.z > 1.0f) shadow_sum = 1.0f;
    // AMBIENT_SH (render_geometry.comp:40-57): only sh[0] = sh[2] = 0.025.
    if (u.debug != 0 && u.debug != 4) {
        const f3 o = debug_view(u.debug, base, ci, tri, f.views[0].refs[slot].meshlet_index, normal);
        store_hdr(f.hdr, f.hdr_half, pix, o.x, o.y, o.z);
        return;
    }
    // The reference's 9-term sum has zero coefficients but sh[0] and sh[2]:
    // for a finite normal each zero term is +-0, and adding +-0 leaves a sum
    // unchanged, so the sum is bit for bit sh0 + sh0 * n.y.
    const float amb_level = 0.025f;
    const f3 sh0{amb_level, amb_level, amb_level};
    f3 amb = sh0 + sh0 * normal.y;
    f3 ambient = amb * (base * (1.0f - metallic));
    float sun_intensity = kPi * shadow_sum;
    // Uniforms.sun_intensity is the light colour (1,1,1 in the reference, whose
    // shaders never read it; main.cpp:649): a multiply by 1 leaves every bit.
    f3 sun = (BRDF(view_vector, ld3(u.sun_dir), normal, roughness, metallic, base, alpha) * sun_intensity) *
             ld3(u.sun_intensity);
    f3 o = sun + ambient;
    if (u.debug == 4) o = clock_view(*clock_slot);
    store_hdr(f.hdr, f.hdr_half, pix, o.x, o.y, o.z);
}

#ifndef LH_RESOLVE_MIN_BLOCKS
#define LH_RESOLVE_MIN_BLOCKS 3
#endif
constexpr uint32_t kResolveWarps = 8;   // warps per block = rows of a strip
constexpr uint32_t kStripCols = 128;    // a strip: 128 x 8 pixels (4 tiles of 32 x 8)
#ifndef LH_RESOLVE_STAGES
#define LH_RESOLVE_STAGES 2
#endif
constexpr uint32_t kResolveStages = LH_RESOLVE_STAGES;  // strips in flight per warp (build knob)

// One thread per pixel over 128 x 8-pixel strips, one warp per strip row
// (four 32-pixel steps); a grid of resident blocks strides over the strips,
// so a block's warps shade the 8 rows of one strip together and their
// gathers stay close in 2D.  With kTma each warp stages the visibility words
// of its row of its next kResolveStages strips in shared memory with TMA row
// loads (box 128 x 1 = 1 KB, one mbarrier per stage) issued by its lane 0;
// nothing synchronises beyond the warp.  Without (rows not 16-byte aligned)
// each thread loads its own words.
template <bool kTma>
__global__ void __launch_bounds__(kResolveWarps * 32, LH_RESOLVE_MIN_BLOCKS)
    k_resolve(FrameDev f, const __grid_constant__ CUtensorMap vis_map, uint32_t strips_x, uint32_t n_strips) {
    __shared__ __align__(128) unsigned long long s_vis[kResolveWarps][kResolveStages][kStripCols];
    __shared__ __align__(8) uint64_t s_bar[kResolveWarps][kResolveStages];
    pdl_enter();
    __shared__ long long s_clock[kResolveWarps][32];
    __shared__ uint32_t s_keys[kResolveWarps][kShareTris];
    __shared__ __align__(16) lh_mat4 s_uvs[4];
    __shared__ __align__(16) float4 s_vert[kResolveWarps][3 * 3 * kShareTris];
    const uint32_t W = f.uniforms->window_size.x, H = f.uniforms->window_size.y;
    const uint32_t lane = threadIdx.x, warp = threadIdx.y;
    // the cascades' matrices, read by every pixel's cascade selection
    if (warp < 2) {  // 64 floats
        const float* src = &f.misc->uv_space_shadow_matrices[0].cols[0].x;
        reinterpret_cast<float*>(s_uvs)[warp * 32 + lane] = src[warp * 32 + lane];
    }
    __syncthreads();
    unsigned long long(*vis_buf)[kStripCols] = s_vis[warp];
    uint64_t* bar = s_bar[warp];
    constexpr uint32_t kRowBytes = kStripCols * 8;
    // the warp's row of strip `t` and whether it holds pixels
    auto row_of = [&](uint32_t t, int32_t& x0, int32_t& y) {
        x0 = (int32_t)((t % strips_x) * kStripCols);
        y = (int32_t)((t / strips_x) * kResolveWarps + warp);
        return (uint32_t)y < H;
    };
    if (kTma) {
        if (lane == 0) {
            for (uint32_t k = 0; k < kResolveStages; k++) mbar_init(&bar[k], 1);
            mbar_init_fence();
            for (uint32_t k = 0; k < kResolveStages; k++) {
                const uint32_t t = blockIdx.x + k * gridDim.x;
                int32_t x0, y;
                if (t >= n_strips) break;
                if (!row_of(t, x0, y)) continue;
                mbar_expect_tx(&bar[k], kRowBytes);
                tma_load_2d(vis_buf[k], &vis_map, x0, y, &bar[k]);
            }
        }
        __syncwarp();
    }
    uint32_t k = 0;
    uint32_t prev_slots = 0;  // the vertex slots of the warp's last row segment
    const float rcp_w = 1.0f / (float)W;
    for (uint32_t t = blockIdx.x; t < n_strips; t += gridDim.x, k++) {
        int32_t x0, y;
        if (!row_of(t, x0, y)) continue;  // below the image (last strip row): no load was issued
        const uint32_t st = k % kResolveStages;
        if (kTma) {
            const bool ok = mbar_wait(&bar[st], (k / kResolveStages) & 1u);
            if (__any_sync(0xFFFFFFFFu, !ok)) {
                // a copy that never landed: report it, wait (bounded) for the
                // warp's other copies in flight, and stop this warp
                if (lane == 0) {
                    atomicOr(&f.status[kStFlags], LH_FLAG_TIMEOUT);
                    for (uint32_t j = 1; j < kResolveStages; j++) {
                        const uint32_t kk = k + j, tt = t + j * gridDim.x;
                        int32_t xx, yy;
                        if (tt >= n_strips) break;
                        if (row_of(tt, xx, yy)) mbar_wait(&bar[kk % kResolveStages], (kk / kResolveStages) & 1u);
                    }
                }
                break;
            }
        }
        const float ndc_y = (float)y / (float)H * 2.0f - 1.0f;
#pragma unroll 1
        for (uint32_t j = 0; j < kStripCols / 32; j++) {
            const uint32_t x = (uint32_t)x0 + 32 * j + lane;
            const bool in_view = x < W;  // every lane takes part: the vertex stage is a warp collective
            const unsigned long long vis =
                !in_view ? 0ull
                         : kTma ? vis_buf[st][32 * j + lane]
                                : __ldcs(reinterpret_cast<const unsigned long long*>(f.visibility) + (size_t)y * W + x);
            resolve_pixel(f, x, (uint32_t)y, vis, in_view, &s_clock[warp][lane], s_keys[warp], s_vert[warp], prev_slots,
                          s_uvs, rcp_w, ndc_y);
        }
        if (kTma) {
            __syncwarp();  // stage st is free again; the other stage's strip is already in flight
            const uint32_t next = t + kResolveStages * gridDim.x;
            int32_t nx0, ny;
            if (lane == 0 && next < n_strips && row_of(next, nx0, ny)) {
                mbar_expect_tx(&bar[st], kRowBytes);
                tma_load_2d(vis_buf[st], &vis_map, nx0, ny, &bar[st]);
            }
        }
    }
}

// grid = (blocks, n_views), or (blocks, 1) without `targets`.  With
// `has_start`, view 0's blocks also zero the frame's scratch and block (0, 0)
// stores the frame's uniforms and constants (nothing in this kernel reads
// either).  Without `targets` only block (0, 0) resets the per-view counters
// and the depth range: the targets are cleared by the instance-cull launches
// (launch_cull_instances with `clear`), beside the cull.
__global__ void __launch_bounds__(256) k_clear_targets(FrameDev f, const __grid_constant__ FrameStart start,
                                                       uint32_t has_start, uint32_t targets) {
    pdl_enter();
    if (has_start && blockIdx.y == 0) {
        const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t i = tid; i < start.reset_words; i += stride) start.reset[i] = make_uint4(0u, 0u, 0u, 0u);
        if (blockIdx.x == 0) {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&start.u);
            uint32_t* dst = reinterpret_cast<uint32_t*>(start.d_uniforms);
            for (uint32_t i = threadIdx.x; i < sizeof(Uniforms) / 4; i += blockDim.x) dst[i] = src[i];
            if (threadIdx.x < 2) start.d_consts[threadIdx.x] = start.consts[threadIdx.x];
        }
    }
    if (targets)
        phase_clear_view(f, blockIdx.y, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                         (uint64_t)gridDim.x * blockDim.x, blockIdx.x == 0 && blockIdx.y == 0);
    else if (blockIdx.x == 0)
        reset_view_counters(f);
}

// Depth reduction; the last block to finish fits the cascades.
__global__ void __launch_bounds__(256) k_depth_reduce_fit(FrameDev f) {
    pdl_enter();
    phase_depth_reduce(f, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x);
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&f.status[kStReduceDone], 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) phase_fit(f);
}

}  // namespace

namespace {
__global__ void __launch_bounds__(256) k_linearize_texture(const uchar4* src, float4* dst, size_t n, uint32_t srgb,
                                                           const float* lut) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uchar4 p = src[i];
        float4 o;
        if (srgb) {
            o.x = lut[p.x];
            o.y = lut[p.y];
            o.z = lut[p.z];
        } else {
            o.x = (float)p.x / 255.0f;
            o.y = (float)p.y / 255.0f;
            o.z = (float)p.z / 255.0f;
        }
        o.w = (float)p.w / 255.0f;
        dst[i] = o;
    }
}
}  // namespace

cudaError_t launch_linearize_texture(const uchar4* src, float4* dst, size_t n, uint32_t srgb, const float* lut,
                                     cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const size_t blocks = std::min<size_t>((n + 255) / 256, 4096);
    k_linearize_texture<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n, srgb, lut);
    return cudaGetLastError();
}

cudaError_t launch_clear_targets(const FrameDev& f, cudaStream_t s, int sms, const FrameStart* start, bool targets) {
    const dim3 grid((unsigned)sms, targets ? f.n_views : 1u);
    if (start) return launch_pdl(k_clear_targets, grid, dim3(256), s, f, *start, 1u, targets ? 1u : 0u);
    FrameStart none;
    std::memset(&none, 0, sizeof(none));
    return launch_pdl(k_clear_targets, grid, dim3(256), s, f, none, 0u, targets ? 1u : 0u);
}

// The frame-start kernel node of a captured graph, and its parameters set
// for the next replay: the uniforms, constants and scratch reset ride on the
// replay's kernel parameters instead of a host-to-device copy before it.
bool is_clear_targets_node(cudaGraphNode_t node) {
    cudaGraphNodeType type;
    if (cudaGraphNodeGetType(node, &type) != cudaSuccess || type != cudaGraphNodeTypeKernel) return false;
    cudaKernelNodeParams p = {};
    if (cudaGraphKernelNodeGetParams(node, &p) != cudaSuccess) return false;
    return p.func == reinterpret_cast<void*>(k_clear_targets);
}
cudaError_t set_clear_targets_node(cudaGraphExec_t exec, cudaGraphNode_t node, const FrameDev& f, int sms,
                                   const FrameStart& start) {
    FrameDev fa = f;
    FrameStart sa = start;
    uint32_t has_start = 1u, targets = 0u;
    void* args[4] = {&fa, &sa, &has_start, &targets};
    cudaKernelNodeParams p = {};
    p.func = reinterpret_cast<void*>(k_clear_targets);
    p.gridDim = dim3((unsigned)sms, 1u);
    p.blockDim = dim3(256);
    p.sharedMemBytes = 0;
    p.kernelParams = args;
    p.extra = nullptr;
    return cudaGraphExecKernelNodeSetParams(exec, node, &p);
}

cudaError_t launch_depth_reduce_fit(const FrameDev& f, cudaStream_t s, int sms) {
    return launch_pdl(k_depth_reduce_fit, dim3((unsigned)sms * 2), dim3(256), s, f);
}

cudaError_t launch_resolve(const FrameDev& f, uint32_t width, uint32_t height, const CUtensorMap* vis_map,
                           cudaStream_t s, int sms) {
    const uint32_t strips_x = (width + kStripCols - 1) / kStripCols, strips_y = (height + kResolveWarps - 1) / kResolveWarps;
    const uint32_t n_strips = strips_x * strips_y;
    if (n_strips == 0) return cudaSuccess;
    const uint32_t grid = std::min<uint32_t>(n_strips, (uint32_t)sms * LH_RESOLVE_MIN_BLOCKS);
#ifdef LH_RESOLVE_NO_TMA
    vis_map = nullptr;  // comparison builds: per-thread loads of the visibility words
#endif
    if (vis_map) return launch_pdl(k_resolve<true>, dim3(grid), dim3(32, kResolveWarps), s, f, *vis_map, strips_x, n_strips);
    CUtensorMap none;
    std::memset(&none, 0, sizeof(none));
    return launch_pdl(k_resolve<false>, dim3(grid), dim3(32, kResolveWarps), s, f, none, strips_x, n_strips);
}

}  // namespace lh
