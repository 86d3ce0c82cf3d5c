// Lighting of one visibility-buffer pixel and its hand-written adjoint.
//
// The forward follows render_geometry.comp:126-266 (barycentrics from
// vbuffer.glsl:11-63, interpolation, view vector, normal, cascade PCF,
// materials, SH ambient, BRDF from pbr.glsl:44-96) in the same operation
// order as the resolve kernel.  `shade()` recomputes that forward from the
// pixel's three vertices (visibility is held fixed: the triangle, the
// back-face flip, the cascade and every shadow-map compare result are the
// forward's) and then runs the reverse pass, returning d(loss)/d(input) for
//   - the three vertices' world positions (then M^T to mesh space by the caller),
//   - their raw normals and raw uvs,
//   - the base-colour factor, the 4 base-colour texels and the 4
//     metallic-roughness texels the bilinear samples used,
//   - the light direction and the light colour.
// Normal-mapped materials are shaded but not differentiated (flag in the
// result).  Compiled for the device (float) by the backward kernel and for
// the host (double and float) by the CPU derivative checks.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define LH_HD __host__ __device__ __forceinline__
#else
#define LH_HD inline
#endif

namespace lh {
namespace shade {

template <class T> struct v2 { T x, y; };
template <class T> struct v3 { T x, y, z; };

template <class T> LH_HD v3<T> add(v3<T> a, v3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> LH_HD v3<T> sub(v3<T> a, v3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> LH_HD v3<T> mul(v3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> LH_HD v3<T> mulv(v3<T> a, v3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> LH_HD T dot(v3<T> a, v3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> LH_HD v3<T> neg(v3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> LH_HD v3<T> cross(v3<T> a, v3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

LH_HD float tsqrt(float x) { return sqrtf(x); }
LH_HD double tsqrt(double x) { return sqrt(x); }
LH_HD float tpow(float a, float b) { return powf(a, b); }
LH_HD double tpow(double a, double b) { return pow(a, b); }
LH_HD float tfloor(float a) { return floorf(a); }
LH_HD double tfloor(double a) { return floor(a); }
LH_HD float tabs(float a) { return fabsf(a); }
LH_HD double tabs(double a) { return fabs(a); }
template <class T> LH_HD T tmax(T a, T b) { return (a < b) ? b : a; }
template <class T> LH_HD T tmin(T a, T b) { return (b < a) ? b : a; }
template <class T> LH_HD T tclamp(T x, T lo, T hi) { return tmin(tmax(x, lo), hi); }
// derivative of clamp: 1 strictly inside the interval
template <class T> LH_HD T dclamp(T x, T lo, T hi) { return (x > lo && x < hi) ? T(1) : T(0); }

template <class T> LH_HD v3<T> normalize(v3<T> v) {
    T l = tsqrt(dot(v, v));
    return {v.x / l, v.y / l, v.z / l};
}
// reverse of y = normalize(x): gx = (gy - y (y . gy)) / |x|
template <class T> LH_HD v3<T> normalize_adj(v3<T> x, v3<T> y, v3<T> gy) {
    T l = tsqrt(dot(x, x));
    T d = dot(y, gy);
    return {(gy.x - y.x * d) / l, (gy.y - y.y * d) / l, (gy.z - y.z * d) / l};
}

// Column-major 4x4 (m[c][r]) applied to (v, w).
template <class T> LH_HD v3<T> xform3(const float m[4][4], v3<T> v, T w) {
    return {((T(m[0][0]) * v.x + T(m[1][0]) * v.y) + T(m[2][0]) * v.z) + T(m[3][0]) * w,
            ((T(m[0][1]) * v.x + T(m[1][1]) * v.y) + T(m[2][1]) * v.z) + T(m[3][1]) * w,
            ((T(m[0][2]) * v.x + T(m[1][2]) * v.y) + T(m[2][2]) * v.z) + T(m[3][2]) * w};
}
template <class T> LH_HD T xform_w(const float m[4][4], v3<T> v, T w) {
    return ((T(m[0][3]) * v.x + T(m[1][3]) * v.y) + T(m[2][3]) * v.z) + T(m[3][3]) * w;
}

// One bilinear sample: the 4 texels (linear values) and the weights' inputs.
template <class T> struct Bilinear {
    T t00[4], t10[4], t01[4], t11[4];
    T a, b;          // fractional position
    T size_u, size_v;  // texture size (d(frac)/d(uv))
    int32_t i0, i1, j0, j1;  // texel coordinates (wrapped)
    uint32_t index;
};
template <class T> LH_HD T bilerp(const Bilinear<T>& s, int c) {
    T w00 = (T(1) - s.a) * (T(1) - s.b), w10 = s.a * (T(1) - s.b), w01 = (T(1) - s.a) * s.b, w11 = s.a * s.b;
    return ((s.t00[c] * w00 + s.t10[c] * w10) + s.t01[c] * w01) + s.t11[c] * w11;
}

// Fixed (non-differentiated) inputs of a pixel.
struct PixelFixed {
    float pv[4][4];        // combined_perspective_view
    float nt[3][3];        // normal_transform, column major
    float uvs[4][4];       // uv_space_shadow_matrices[cascade] (cascade selected by the forward)
    float cam[3];
    float ndc[2];
    float win[2];
    float ts[2], toff[2];  // texture scale / offset
    float bias;            // shadow bias (alpha clip)
    float shadow_size;
    uint32_t cascade;      // 0..4 (4 = fell through: layer 3)
    uint32_t thin;         // alpha clip: thin-walled lobe
    uint32_t base_tex, mr_tex;
    uint32_t has_normal_map;
    // discrete decisions of the forward, held fixed (see decide())
    float flip;              // +1, or -1 when the triangle is seen from behind
    uint32_t shadow_const;   // shadow coordinate beyond the cascade's far plane
    uint64_t cmp;            // 36 shadow-map compare results: bit 4*tap + texel
};

// Differentiated inputs.
template <class T> struct PixelParams {
    v3<T> W[3];   // world positions of the vertices
    v3<T> N[3];   // raw normals
    v2<T> UV[3];  // raw uvs
    v3<T> bcf;    // base colour factor
    v3<T> sun;    // light direction
    v3<T> light;  // light colour (1,1,1 reproduces the reference)
};

template <class T> struct PixelGrad {
    v3<T> W[3], N[3];
    v2<T> UV[3];
    v3<T> bcf, sun, light;
    T base_texel[4][3];  // d/d(linear rgb) of texels 00, 10, 01, 11
    T mr_texel[4][2];    // d/d(roughness = g, metallic = b) of the 4 texels
    int32_t base_ij[4], mr_ij[4];  // texel columns (i0, i1) and rows (j0, j1) of the two samples
    uint32_t base_index, mr_index;
    bool differentiated;
};

// Shadow-map access for the PCF: compare result of texel (i, j) of the layer
// against `ref` (1 when ref < stored).
// Compare results of one PCF tap (4 bits: texels 00, 10, 01, 11).
template <class T, class Sampler>
LH_HD uint32_t pcf_bits(const Sampler& smp, uint32_t layer, T u, T v, T ref, T S) {
    T uu = u * S - T(0.5), vv = v * S - T(0.5);
    if (!(tabs(uu) < T(1e9))) uu = T(0);
    if (!(tabs(vv) < T(1e9))) vv = T(0);
    // |uu|, |vv| < 1e9: 32-bit texel coordinates suffice
    int32_t i0 = (int32_t)tfloor(uu), j0 = (int32_t)tfloor(vv);
    return (smp.shadow_cmp(layer, i0, j0, ref) != T(0) ? 1u : 0u) |
           (smp.shadow_cmp(layer, i0 + 1, j0, ref) != T(0) ? 2u : 0u) |
           (smp.shadow_cmp(layer, i0, j0 + 1, ref) != T(0) ? 4u : 0u) |
           (smp.shadow_cmp(layer, i0 + 1, j0 + 1, ref) != T(0) ? 8u : 0u);
}

// One PCF tap with fixed compare results `bits`: the bilinear weights and
// their derivatives in the tap's fractional position.
template <class T>
LH_HD T pcf_tap(uint32_t bits, T u, T v, T S, T& da, T& db) {
    T uu = u * S - T(0.5), vv = v * S - T(0.5);
    if (!(tabs(uu) < T(1e9))) uu = T(0);
    if (!(tabs(vv) < T(1e9))) vv = T(0);
    T fu = tfloor(uu), fv = tfloor(vv);
    T a = uu - fu, b = vv - fv;
    T c00 = (bits & 1u) ? T(1) : T(0), c10 = (bits & 2u) ? T(1) : T(0);
    T c01 = (bits & 4u) ? T(1) : T(0), c11 = (bits & 8u) ? T(1) : T(0);
    T w00 = (T(1) - a) * (T(1) - b), w10 = a * (T(1) - b), w01 = (T(1) - a) * b, w11 = a * b;
    da = (T(1) - b) * (c10 - c00) + b * (c11 - c01);
    db = (T(1) - a) * (c01 - c00) + a * (c11 - c10);
    return ((c00 * w00 + c10 * w10) + c01 * w01) + c11 * w11;
}

template <class T> struct BurleyOut { T value, dNoV, dNoL, dLoH, da; };
// Fd_Burley (pbr.glsl:8-13) and its partial derivatives.
template <class T> LH_HD BurleyOut<T> burley(T NoV, T NoL, T LoH, T a) {
    const T PI = T(3.14159265358979323846f);
    T f90 = T(0.5) + T(2) * a * LoH * LoH;
    T ql = tpow(T(1) - NoL, T(5)), qv = tpow(T(1) - NoV, T(5));
    T light = T(1) + (f90 - T(1)) * ql;
    T view = T(1) + (f90 - T(1)) * qv;
    BurleyOut<T> r;
    r.value = light * view * (T(1) / PI);
    T dl_dNoL = -(f90 - T(1)) * T(5) * tpow(T(1) - NoL, T(4));
    T dv_dNoV = -(f90 - T(1)) * T(5) * tpow(T(1) - NoV, T(4));
    T dval_df90 = (ql * view + light * qv) / PI;
    r.dNoL = dl_dNoL * view / PI;
    r.dNoV = light * dv_dNoV / PI;
    r.dLoH = dval_df90 * T(4) * a * LoH;
    r.da = dval_df90 * T(2) * LoH * LoH;
    return r;
}

// The forward's discrete decisions for `p` (face flip, far-plane test,
// the 36 compare results), in the arithmetic of the inputs given.
template <class T, class Sampler>
LH_HD void decide(PixelFixed& fx, const PixelParams<T>& p, const Sampler& smp) {
    v3<T> C[3];
    T iw[3];
    v2<T> n[3];
    for (int k = 0; k < 3; k++) {
        C[k] = xform3(fx.pv, p.W[k], T(1));
        iw[k] = T(1) / xform_w(fx.pv, p.W[k], T(1));
        n[k] = {C[k].x * iw[k], C[k].y * iw[k]};
    }
    v2<T> ca{n[2].x - n[1].x, n[2].y - n[1].y}, cb{n[0].x - n[1].x, n[0].y - n[1].y};
    T invDet = T(1) / (ca.x * cb.y - cb.x * ca.y);
    T dxr[3] = {n[1].y - n[2].y, n[2].y - n[0].y, n[0].y - n[1].y};
    T dyr[3] = {n[2].x - n[1].x, n[0].x - n[2].x, n[1].x - n[0].x};
    T ddx0[3], ddy0[3];
    for (int k = 0; k < 3; k++) {
        ddx0[k] = dxr[k] * invDet * iw[k];
        ddy0[k] = dyr[k] * invDet * iw[k];
    }
    T sx = (ddx0[0] * T(1) + ddx0[1] * T(1)) + ddx0[2] * T(1);
    T sy = (ddy0[0] * T(1) + ddy0[1] * T(1)) + ddy0[2] * T(1);
    v2<T> dv{T(fx.ndc[0]) - n[0].x, T(fx.ndc[1]) - n[0].y};
    T wi = T(1) / ((iw[0] + dv.x * sx) + dv.y * sy);
    T lam[3] = {wi * ((iw[0] + dv.x * ddx0[0]) + dv.y * ddy0[0]), wi * ((T(0) + dv.x * ddx0[1]) + dv.y * ddy0[1]),
                wi * ((T(0) + dv.x * ddx0[2]) + dv.y * ddy0[2])};
    v3<T> world = {(p.W[0].x * lam[0] + p.W[1].x * lam[1]) + p.W[2].x * lam[2],
                   (p.W[0].y * lam[0] + p.W[1].y * lam[1]) + p.W[2].y * lam[2],
                   (p.W[0].z * lam[0] + p.W[1].z * lam[1]) + p.W[2].z * lam[2]};
    v3<T> V = normalize(sub(v3<T>{T(fx.cam[0]), T(fx.cam[1]), T(fx.cam[2])}, world));
    v3<T> gn = cross(sub(p.W[1], p.W[0]), sub(p.W[2], p.W[0]));
    fx.flip = dot(gn, V) < T(0) ? -1.0f : 1.0f;
    v3<T> sc = xform3(fx.uvs, world, T(1));
    T scw = xform_w(fx.uvs, world, T(1));
    sc = {sc.x / scw, sc.y / scw, sc.z / scw};
    fx.shadow_const = sc.z > T(1) ? 1u : 0u;
    const uint32_t layer = fx.cascade > 3 ? 3u : fx.cascade;
    uint64_t bits = 0;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = -1; oy <= 1; oy++) {
            const uint32_t tap = (uint32_t)((ox + 1) * 3 + (oy + 1));
            bits |= (uint64_t)pcf_bits(smp, layer, sc.x + T(ox) / T(1024), sc.y + T(oy) / T(1024), sc.z - T(fx.bias),
                                       T(fx.shadow_size))
                    << (4 * tap);
        }
    fx.cmp = bits;
}

// Forward (into *out) and, when `g` is non-null, the reverse pass for the
// upstream gradient `gout` of the pixel's RGB, with the discrete decisions
// in `fx` (decide()) held fixed.  The geometry may be given relative to any
// origin (fx.pv, fx.uvs and fx.cam expressed for the same origin): the
// backward kernel uses the camera, which keeps float32 from cancelling
// world-scale coordinates.  `smp` provides sample(tex, uv) -> Bilinear.
template <class T, class Sampler>
LH_HD void shade(const PixelFixed& fx, const PixelParams<T>& p, const Sampler& smp, v3<T>* out, v3<T> gout,
                 PixelGrad<T>* g) {
    const T PI = T(3.14159265358979323846f);
    // ---- forward
    // clip positions and CalcFullBary (lambda only; the screen derivatives
    // only feed the normal map, which is not differentiated)
    v3<T> C[3];
    T Cw[3], iw[3];
    v2<T> n[3];
    for (int k = 0; k < 3; k++) {
        C[k] = xform3(fx.pv, p.W[k], T(1));
        Cw[k] = xform_w(fx.pv, p.W[k], T(1));
        iw[k] = T(1) / Cw[k];
        n[k] = {C[k].x * iw[k], C[k].y * iw[k]};
    }
    v2<T> ca{n[2].x - n[1].x, n[2].y - n[1].y}, cb{n[0].x - n[1].x, n[0].y - n[1].y};
    T det = ca.x * cb.y - cb.x * ca.y;
    T invDet = T(1) / det;
    T dxr[3] = {n[1].y - n[2].y, n[2].y - n[0].y, n[0].y - n[1].y};
    T dyr[3] = {n[2].x - n[1].x, n[0].x - n[2].x, n[1].x - n[0].x};
    T ddx0[3], ddy0[3];
    for (int k = 0; k < 3; k++) {
        ddx0[k] = dxr[k] * invDet * iw[k];
        ddy0[k] = dyr[k] * invDet * iw[k];
    }
    T sx = (ddx0[0] * T(1) + ddx0[1] * T(1)) + ddx0[2] * T(1);
    T sy = (ddy0[0] * T(1) + ddy0[1] * T(1)) + ddy0[2] * T(1);
    v2<T> dv{T(fx.ndc[0]) - n[0].x, T(fx.ndc[1]) - n[0].y};
    T iiw = (iw[0] + dv.x * sx) + dv.y * sy;
    T wi = T(1) / iiw;
    T av[3] = {(iw[0] + dv.x * ddx0[0]) + dv.y * ddy0[0], (T(0) + dv.x * ddx0[1]) + dv.y * ddy0[1],
               (T(0) + dv.x * ddx0[2]) + dv.y * ddy0[2]};
    T lam[3] = {wi * av[0], wi * av[1], wi * av[2]};
    // interpolation (InterpolateWithDeriv value: dot(v, lambda))
    v3<T> world = {(p.W[0].x * lam[0] + p.W[1].x * lam[1]) + p.W[2].x * lam[2],
                   (p.W[0].y * lam[0] + p.W[1].y * lam[1]) + p.W[2].y * lam[2],
                   (p.W[0].z * lam[0] + p.W[1].z * lam[1]) + p.W[2].z * lam[2]};
    v2<T> uvs[3];
    for (int k = 0; k < 3; k++) uvs[k] = {p.UV[k].x * T(fx.ts[0]), p.UV[k].y * T(fx.ts[1])};
    v2<T> uv = {((uvs[0].x * lam[0] + uvs[1].x * lam[1]) + uvs[2].x * lam[2]) + T(fx.toff[0]),
                ((uvs[0].y * lam[0] + uvs[1].y * lam[1]) + uvs[2].y * lam[2]) + T(fx.toff[1])};
    v3<T> cam{T(fx.cam[0]), T(fx.cam[1]), T(fx.cam[2])};
    v3<T> vd = sub(cam, world);
    v3<T> V = normalize(vd);
    v3<T> nk[3];
    for (int k = 0; k < 3; k++) nk[k] = normalize(p.N[k]);
    v3<T> ni = {(nk[0].x * lam[0] + nk[1].x * lam[1]) + nk[2].x * lam[2],
                (nk[0].y * lam[0] + nk[1].y * lam[1]) + nk[2].y * lam[2],
                (nk[0].z * lam[0] + nk[1].z * lam[1]) + nk[2].z * lam[2]};
    v3<T> nt = {(T(fx.nt[0][0]) * ni.x + T(fx.nt[1][0]) * ni.y) + T(fx.nt[2][0]) * ni.z,
                (T(fx.nt[0][1]) * ni.x + T(fx.nt[1][1]) * ni.y) + T(fx.nt[2][1]) * ni.z,
                (T(fx.nt[0][2]) * ni.x + T(fx.nt[1][2]) * ni.y) + T(fx.nt[2][2]) * ni.z};
    v3<T> n0 = normalize(nt);
    const T flip = T(fx.flip);
    v3<T> normal = mul(n0, flip);
    // shadow: cascade fixed by the forward; PCF weights differentiable
    v3<T> sc = xform3(fx.uvs, world, T(1));
    T scw = xform_w(fx.uvs, world, T(1));
    sc = {sc.x / scw, sc.y / scw, sc.z / scw};
    T shadow = T(0), dsh_dx = T(0), dsh_dy = T(0);
    const T S = T(fx.shadow_size);
    const bool shadow_const = fx.shadow_const != 0;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = -1; oy <= 1; oy++) {
            T da, db;
            const uint32_t tap = (uint32_t)((ox + 1) * 3 + (oy + 1));
            shadow += pcf_tap((uint32_t)(fx.cmp >> (4 * tap)) & 15u, sc.x + T(ox) / T(1024), sc.y + T(oy) / T(1024), S,
                              da, db);
            dsh_dx += da * S;
            dsh_dy += db * S;
        }
    shadow /= T(9);
    dsh_dx /= T(9);
    dsh_dy /= T(9);
    if (shadow_const) shadow = T(1);
    // materials
    Bilinear<T> sb = smp.sample(fx.base_tex, uv), sm = smp.sample(fx.mr_tex, uv);
    v3<T> texc{bilerp(sb, 0), bilerp(sb, 1), bilerp(sb, 2)};
    v3<T> base = mulv(texc, p.bcf);
    T rough = bilerp(sm, 1), metal = bilerp(sm, 2);
    // (a normal map would replace `normal` here; not differentiated)
    // SH ambient: only sh[0] = sh[2] = 0.025 are non-zero
    const T amb_level = T(0.025f);
    T amb = amb_level + amb_level * normal.y;
    v3<T> diffuse = mul(base, T(1) - metal);
    v3<T> ambient = mul(diffuse, amb);
    // BRDF (pbr.glsl:44-96)
    v3<T> L = p.sun;
    v3<T> h0 = add(V, L);
    v3<T> H = normalize(h0);
    T refl = (T(1.5) - T(1)) / (T(1.5) + T(1));
    refl = refl * refl;
    v3<T> f0 = add(mul(v3<T>{refl, refl, refl}, T(1) - metal), mul(base, metal));
    T NoVr = dot(normal, V), NoLr = dot(normal, L), NoHr = dot(normal, H), LoHr = dot(L, H);
    T NoV = tclamp(NoVr, T(1e-5f), T(1)), NoL = tclamp(NoLr, T(0), T(1));
    T NoH = tclamp(NoHr, T(0), T(1)), LoH = tclamp(LoHr, T(0), T(1));
    T a = rough * rough;
    T a2 = a * a;
    T fq = (NoH * a2 - NoH) * NoH + T(1);
    T D = a2 / (PI * fq * fq);
    T q5 = tpow(T(1) - LoH, T(5));
    v3<T> F{f0.x + (T(1) - f0.x) * q5, f0.y + (T(1) - f0.y) * q5, f0.z + (T(1) - f0.z) * q5};
    T sL = tsqrt((-NoL * a2 + NoL) * NoL + a2), sV = tsqrt((-NoV * a2 + NoV) * NoV + a2);
    T GGXL = NoV * sL, GGXV = NoL * sV;
    T Vis = T(0.5) / (GGXV + GGXL);
    BurleyOut<T> fb = burley(NoV, NoL, LoH, a);
    v3<T> pre{(diffuse.x * fb.value + F.x * (D * Vis)) * NoL, (diffuse.y * fb.value + F.y * (D * Vis)) * NoL,
              (diffuse.z * fb.value + F.z * (D * Vis)) * NoL};
    v3<T> irr{tmax(pre.x, T(0)), tmax(pre.y, T(0)), tmax(pre.z, T(0))};
    T rNoVr = dot(neg(normal), V), rNoLr = dot(neg(normal), L);
    T rNoV = tclamp(rNoVr, T(1e-5f), T(1)), rNoL = tclamp(rNoLr, T(0), T(1));
    BurleyOut<T> fr = burley(rNoV, rNoL, LoH, a);
    if (fx.thin) irr = add(irr, mul(diffuse, fr.value * rNoL));
    bool nanc[3] = {irr.x != irr.x, irr.y != irr.y, irr.z != irr.z};
    if (nanc[0]) irr.x = T(0);
    if (nanc[1]) irr.y = T(0);
    if (nanc[2]) irr.z = T(0);
    T sun_scale = PI * shadow;
    v3<T> light = p.light;
    v3<T> sun = mulv(mul(irr, sun_scale), light);
    *out = add(sun, ambient);
    if (!g) return;

    // ---- reverse
    g->differentiated = fx.has_normal_map == 0;
    // sun = irr * (pi * shadow) * light
    v3<T> g_irr{gout.x * sun_scale * light.x, gout.y * sun_scale * light.y, gout.z * sun_scale * light.z};
    g->light = {gout.x * irr.x * sun_scale, gout.y * irr.y * sun_scale, gout.z * irr.z * sun_scale};
    T g_shadow = PI * ((gout.x * irr.x * light.x + gout.y * irr.y * light.y) + gout.z * irr.z * light.z);
    if (nanc[0]) g_irr.x = T(0);
    if (nanc[1]) g_irr.y = T(0);
    if (nanc[2]) g_irr.z = T(0);
    v3<T> g_diffuse{T(0), T(0), T(0)}, g_normal{T(0), T(0), T(0)}, g_V{T(0), T(0), T(0)}, g_L{T(0), T(0), T(0)};
    T g_LoH = T(0), g_a = T(0);
    // thin-walled lobe: diffuse * Fd(rNoV, rNoL) * rNoL
    if (fx.thin) {
        T dsum = (g_irr.x * diffuse.x + g_irr.y * diffuse.y) + g_irr.z * diffuse.z;
        g_diffuse = add(g_diffuse, mul(g_irr, fr.value * rNoL));
        T g_rNoL = dsum * (fr.value + fr.dNoL * rNoL) * dclamp(rNoLr, T(0), T(1));
        T g_rNoV = dsum * fr.dNoV * rNoL * dclamp(rNoVr, T(1e-5f), T(1));
        g_LoH += dsum * fr.dLoH * rNoL;
        g_a += dsum * fr.da * rNoL;
        // rNoV = dot(-n, V), rNoL = dot(-n, L)
        g_normal = sub(g_normal, add(mul(V, g_rNoV), mul(L, g_rNoL)));
        g_V = sub(g_V, mul(normal, g_rNoV));
        g_L = sub(g_L, mul(normal, g_rNoL));
    }
    v3<T> g_pre{pre.x > T(0) ? g_irr.x : T(0), pre.y > T(0) ? g_irr.y : T(0), pre.z > T(0) ? g_irr.z : T(0)};
    // pre_c = (diffuse_c * Fd + F_c * D * Vis) * NoL
    T DV = D * Vis;
    v3<T> g_F{g_pre.x * DV * NoL, g_pre.y * DV * NoL, g_pre.z * DV * NoL};
    g_diffuse = add(g_diffuse, mul(g_pre, fb.value * NoL));
    T g_fd = ((g_pre.x * diffuse.x + g_pre.y * diffuse.y) + g_pre.z * diffuse.z) * NoL;
    T g_DV = ((g_pre.x * F.x + g_pre.y * F.y) + g_pre.z * F.z) * NoL;
    T g_NoL = (g_pre.x * (diffuse.x * fb.value + F.x * DV) + g_pre.y * (diffuse.y * fb.value + F.y * DV)) +
              g_pre.z * (diffuse.z * fb.value + F.z * DV);
    T g_NoV = T(0), g_NoH = T(0);
    // Burley
    g_NoV += g_fd * fb.dNoV;
    g_NoL += g_fd * fb.dNoL;
    g_LoH += g_fd * fb.dLoH;
    g_a += g_fd * fb.da;
    // DV = D * Vis
    T g_D = g_DV * Vis, g_Vis = g_DV * D;
    // Vis = 0.5 / (GGXV + GGXL)
    T den = GGXV + GGXL;
    T g_den = -g_Vis * T(0.5) / (den * den);
    T g_GGXV = g_den, g_GGXL = g_den;
    // GGXL = NoV * sL, sL = sqrt(NoL^2 (1 - a2) + a2)
    g_NoV += g_GGXL * sL;
    T g_sL = g_GGXL * NoV;
    g_NoL += g_GGXV * sV;
    T g_sV = g_GGXV * NoL;
    T g_a2 = T(0);
    // sL^2 = (-NoL a2 + NoL) NoL + a2
    g_NoL += g_sL / (T(2) * sL) * (T(2) * NoL * (T(1) - a2));
    g_a2 += g_sL / (T(2) * sL) * (T(1) - NoL * NoL);
    g_NoV += g_sV / (T(2) * sV) * (T(2) * NoV * (T(1) - a2));
    g_a2 += g_sV / (T(2) * sV) * (T(1) - NoV * NoV);
    // D = a2 / (pi fq^2), fq = NoH^2 (a2 - 1) + 1
    T g_fq = -g_D * T(2) * a2 / (PI * fq * fq * fq);
    g_a2 += g_D / (PI * fq * fq) + g_fq * NoH * NoH;
    g_NoH += g_fq * T(2) * NoH * (a2 - T(1));
    // F_c = f0_c + (1 - f0_c) q5, q5 = (1 - LoH)^5
    v3<T> g_f0{g_F.x * (T(1) - q5), g_F.y * (T(1) - q5), g_F.z * (T(1) - q5)};
    T g_q5 = (g_F.x * (T(1) - f0.x) + g_F.y * (T(1) - f0.y)) + g_F.z * (T(1) - f0.z);
    g_LoH += -g_q5 * T(5) * tpow(T(1) - LoH, T(4));
    // a2 = a^2, a = rough^2
    g_a += g_a2 * T(2) * a;
    T g_rough = g_a * T(2) * rough;
    // clamps and dots
    g_NoV *= dclamp(NoVr, T(1e-5f), T(1));
    g_NoL *= dclamp(NoLr, T(0), T(1));
    g_NoH *= dclamp(NoHr, T(0), T(1));
    g_LoH *= dclamp(LoHr, T(0), T(1));
    g_normal = add(g_normal, add(add(mul(V, g_NoV), mul(L, g_NoL)), mul(H, g_NoH)));
    g_V = add(g_V, mul(normal, g_NoV));
    g_L = add(g_L, add(mul(normal, g_NoL), mul(H, g_LoH)));
    v3<T> g_H = add(mul(normal, g_NoH), mul(L, g_LoH));
    v3<T> g_h0 = normalize_adj(h0, H, g_H);
    g_V = add(g_V, g_h0);
    g_L = add(g_L, g_h0);
    g->sun = g_L;
    // f0 = refl (1 - metal) + base metal
    v3<T> g_base = mul(g_f0, metal);
    T g_metal = -((g_f0.x * refl + g_f0.y * refl) + g_f0.z * refl) + ((g_f0.x * base.x + g_f0.y * base.y) + g_f0.z * base.z);
    // ambient = diffuse * amb, amb = 0.025 (1 + normal.y)
    g_diffuse = add(g_diffuse, mul(gout, amb));
    g_normal.y += ((gout.x * diffuse.x + gout.y * diffuse.y) + gout.z * diffuse.z) * amb_level;
    // diffuse = base (1 - metal)
    g_base = add(g_base, mul(g_diffuse, T(1) - metal));
    g_metal -= (g_diffuse.x * base.x + g_diffuse.y * base.y) + g_diffuse.z * base.z;
    // base = texc * bcf
    v3<T> g_texc = mulv(g_base, p.bcf);
    g->bcf = mulv(g_base, texc);
    g->base_ij[0] = sb.i0; g->base_ij[1] = sb.i1; g->base_ij[2] = sb.j0; g->base_ij[3] = sb.j1;
    g->mr_ij[0] = sm.i0; g->mr_ij[1] = sm.i1; g->mr_ij[2] = sm.j0; g->mr_ij[3] = sm.j1;
    g->base_index = sb.index;
    g->mr_index = sm.index;
    // texture samples: texel weights and d/duv
    v2<T> g_uv{T(0), T(0)};
    {
        T w[4] = {(T(1) - sb.a) * (T(1) - sb.b), sb.a * (T(1) - sb.b), (T(1) - sb.a) * sb.b, sb.a * sb.b};
        T gt[3] = {g_texc.x, g_texc.y, g_texc.z};
        for (int c = 0; c < 3; c++) {
            for (int q = 0; q < 4; q++) g->base_texel[q][c] = gt[c] * w[q];
            T dda = (T(1) - sb.b) * (sb.t10[c] - sb.t00[c]) + sb.b * (sb.t11[c] - sb.t01[c]);
            T ddb = (T(1) - sb.a) * (sb.t01[c] - sb.t00[c]) + sb.a * (sb.t11[c] - sb.t10[c]);
            g_uv.x += gt[c] * dda * sb.size_u;
            g_uv.y += gt[c] * ddb * sb.size_v;
        }
        T wm[4] = {(T(1) - sm.a) * (T(1) - sm.b), sm.a * (T(1) - sm.b), (T(1) - sm.a) * sm.b, sm.a * sm.b};
        T gm[2] = {g_rough, g_metal};
        for (int c = 0; c < 2; c++) {
            for (int q = 0; q < 4; q++) g->mr_texel[q][c] = gm[c] * wm[q];
            int ch = 1 + c;
            T dda = (T(1) - sm.b) * (sm.t10[ch] - sm.t00[ch]) + sm.b * (sm.t11[ch] - sm.t01[ch]);
            T ddb = (T(1) - sm.a) * (sm.t01[ch] - sm.t00[ch]) + sm.a * (sm.t11[ch] - sm.t10[ch]);
            g_uv.x += gm[c] * dda * sm.size_u;
            g_uv.y += gm[c] * ddb * sm.size_v;
        }
    }
    // shadow: d/d(sc.xy) through the PCF weights, compare results fixed
    v3<T> g_world{T(0), T(0), T(0)};
    if (!shadow_const) {
        T gsx = g_shadow * dsh_dx, gsy = g_shadow * dsh_dy;
        // sc.xy = (UVS (world,1)).xy / w with w = row 3 (constant 1 for the orthographic cascades)
        T gw = -(gsx * sc.x + gsy * sc.y) / scw;
        gsx /= scw;
        gsy /= scw;
        g_world.x += (T(fx.uvs[0][0]) * gsx + T(fx.uvs[0][1]) * gsy) + T(fx.uvs[0][3]) * gw;
        g_world.y += (T(fx.uvs[1][0]) * gsx + T(fx.uvs[1][1]) * gsy) + T(fx.uvs[1][3]) * gw;
        g_world.z += (T(fx.uvs[2][0]) * gsx + T(fx.uvs[2][1]) * gsy) + T(fx.uvs[2][3]) * gw;
    }
    // normal = flip * normalize(nt); nt = NT ni; ni = sum lam_k nk; nk = normalize(N_k)
    v3<T> g_n0 = mul(g_normal, flip);
    v3<T> g_nt = normalize_adj(nt, n0, g_n0);
    v3<T> g_ni{(T(fx.nt[0][0]) * g_nt.x + T(fx.nt[0][1]) * g_nt.y) + T(fx.nt[0][2]) * g_nt.z,
               (T(fx.nt[1][0]) * g_nt.x + T(fx.nt[1][1]) * g_nt.y) + T(fx.nt[1][2]) * g_nt.z,
               (T(fx.nt[2][0]) * g_nt.x + T(fx.nt[2][1]) * g_nt.y) + T(fx.nt[2][2]) * g_nt.z};
    T g_lam[3];
    for (int k = 0; k < 3; k++) {
        g->N[k] = normalize_adj(p.N[k], nk[k], mul(g_ni, lam[k]));
        g_lam[k] = dot(nk[k], g_ni);
    }
    // V = normalize(cam - world)
    g_world = sub(g_world, normalize_adj(vd, V, g_V));
    // uv = sum lam_k uvs_k + offset
    for (int k = 0; k < 3; k++) {
        g->UV[k] = {g_uv.x * lam[k] * T(fx.ts[0]), g_uv.y * lam[k] * T(fx.ts[1])};
        g_lam[k] += g_uv.x * uvs[k].x + g_uv.y * uvs[k].y;
    }
    // world = sum lam_k W_k.  The lambdas sum to 1 for every input, so
    // their gradients may be shifted by a common term: W_k - W_0 instead of
    // W_k keeps float32 from cancelling world-scale coordinates.
    for (int k = 0; k < 3; k++) {
        g->W[k] = mul(g_world, lam[k]);
        g_lam[k] += dot(sub(p.W[k], p.W[0]), g_world);
    }
    // ---- barycentrics: lam_k = wi * av_k
    T g_wi = (g_lam[0] * av[0] + g_lam[1] * av[1]) + g_lam[2] * av[2];
    T g_av[3] = {g_lam[0] * wi, g_lam[1] * wi, g_lam[2] * wi};
    T g_iiw = -g_wi * wi * wi;
    T g_iw[3] = {T(0), T(0), T(0)};
    T g_ddx0[3] = {T(0), T(0), T(0)}, g_ddy0[3] = {T(0), T(0), T(0)};
    v2<T> g_dv{T(0), T(0)};
    g_iw[0] += g_iiw;
    g_dv.x += g_iiw * sx;
    g_dv.y += g_iiw * sy;
    T g_sx = g_iiw * dv.x, g_sy = g_iiw * dv.y;
    g_iw[0] += g_av[0];
    for (int k = 0; k < 3; k++) {
        g_dv.x += g_av[k] * ddx0[k];
        g_dv.y += g_av[k] * ddy0[k];
        g_ddx0[k] += g_av[k] * dv.x + g_sx;
        g_ddy0[k] += g_av[k] * dv.y + g_sy;
    }
    T g_invDet = T(0), g_dxr[3], g_dyr[3];
    for (int k = 0; k < 3; k++) {
        g_dxr[k] = g_ddx0[k] * invDet * iw[k];
        g_dyr[k] = g_ddy0[k] * invDet * iw[k];
        g_invDet += g_ddx0[k] * dxr[k] * iw[k] + g_ddy0[k] * dyr[k] * iw[k];
        g_iw[k] += g_ddx0[k] * dxr[k] * invDet + g_ddy0[k] * dyr[k] * invDet;
    }
    v2<T> g_n[3] = {{-g_dv.x, -g_dv.y}, {T(0), T(0)}, {T(0), T(0)}};
    T g_det = -g_invDet * invDet * invDet;
    v2<T> g_ca{g_det * cb.y, -g_det * cb.x}, g_cb{-g_det * ca.y, g_det * ca.x};
    g_n[2].x += g_ca.x; g_n[2].y += g_ca.y; g_n[1].x -= g_ca.x; g_n[1].y -= g_ca.y;
    g_n[0].x += g_cb.x; g_n[0].y += g_cb.y; g_n[1].x -= g_cb.x; g_n[1].y -= g_cb.y;
    g_n[1].y += g_dxr[0] - g_dxr[2];
    g_n[2].y += g_dxr[1] - g_dxr[0];
    g_n[0].y += g_dxr[2] - g_dxr[1];
    g_n[2].x += g_dyr[0] - g_dyr[1];
    g_n[1].x += g_dyr[2] - g_dyr[0];
    g_n[0].x += g_dyr[1] - g_dyr[2];
    for (int k = 0; k < 3; k++) {
        // n_k = C_k.xy * iw_k, iw_k = 1 / C_k.w
        T gCx = g_n[k].x * iw[k], gCy = g_n[k].y * iw[k];
        g_iw[k] += g_n[k].x * C[k].x + g_n[k].y * C[k].y;
        T gCw = -g_iw[k] * iw[k] * iw[k];
        // C = PV (W, 1): dW_j = sum_r PV[j][r] dC_r  (C.z carries no gradient)
        for (int j = 0; j < 3; j++) {
            T d = (T(fx.pv[j][0]) * gCx + T(fx.pv[j][1]) * gCy) + T(fx.pv[j][3]) * gCw;
            if (j == 0) g->W[k].x += d;
            else if (j == 1) g->W[k].y += d;
            else g->W[k].z += d;
        }
    }
}

}  // namespace shade
}  // namespace lh
