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
//
// The pixel runs in phases so that few values are live at once: geometry
// (barycentrics, interpolants, normal), the PCF shadow term, the surface
// (materials + BRDF) forward and reverse, which hands back d/d(normal, view
// vector, uv, shadow), and the geometry reverse, which recomputes the
// geometry rather than keeping its intermediates alive through the BRDF.
// The fixed matrices are read through accessors (PV, NT, UVS) so that the
// device can keep them in memory instead of registers.
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
LH_HD float tfloor(float a) { return floorf(a); }
LH_HD double tfloor(double a) { return floor(a); }
LH_HD float tabs(float a) { return fabsf(a); }
LH_HD double tabs(double a) { return fabs(a); }
template <class T> LH_HD T tmax(T a, T b) { return (a < b) ? b : a; }
template <class T> LH_HD T tmin(T a, T b) { return (b < a) ? b : a; }
template <class T> LH_HD T tclamp(T x, T lo, T hi) { return tmin(tmax(x, lo), hi); }
// derivative of clamp: 1 strictly inside the interval
template <class T> LH_HD T dclamp(T x, T lo, T hi) { return (x > lo && x < hi) ? T(1) : T(0); }

// IEEE normalize (the forward's decisions use it)
template <class T> LH_HD v3<T> normalize(v3<T> v) {
    T l = tsqrt(dot(v, v));
    return {v.x / l, v.y / l, v.z / l};
}

// Fast arithmetic for the continuous part of shade() (not for decide()): the
// device float instantiation divides and takes square roots approximately
// (div.approx / sqrt.approx, a few ulp -- the gradients are checked at 1e-3
// relative), the host instantiations stay IEEE.  Integer powers multiply.
LH_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdividef(a, b);
#else
    return a / b;
#endif
}
LH_HD double fdiv(double a, double b) { return a / b; }
LH_HD float fsqrt(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return sqrtf(x);
#endif
}
LH_HD double fsqrt(double x) { return sqrt(x); }
template <class T> LH_HD T pow4(T x) {
    const T x2 = x * x;
    return x2 * x2;
}
template <class T> LH_HD T pow5(T x) { return pow4(x) * x; }
template <class T> LH_HD v3<T> fnormalize(v3<T> v) {
    const T r = fdiv(T(1), fsqrt(dot(v, v)));
    return {v.x * r, v.y * r, v.z * r};
}
// reverse of y = normalize(x): gx = (gy - y (y . gy)) / |x|
template <class T> LH_HD v3<T> fnormalize_adj(v3<T> x, v3<T> y, v3<T> gy) {
    const T r = fdiv(T(1), fsqrt(dot(x, x)));
    const T d = dot(y, gy);
    return {(gy.x - y.x * d) * r, (gy.y - y.y * d) * r, (gy.z - y.z * d) * r};
}

// Keeps the device compiler from merging a recomputation with the first
// computation of the same values (a no-op on the host).
LH_HD void opaque(double&) {}
LH_HD void opaque(float& x) {
#if defined(__CUDA_ARCH__)
    asm volatile("" : "+f"(x));
#else
    (void)x;
#endif
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

// What the reverse needs of a bilinear sample, for NC channels from c0:
// the weights' inputs, d(value)/d(a) and d(value)/d(b), the texels.
template <class T, int NC> struct SampleAdj {
    T a, b, size_u, size_v;
    T dda[NC], ddb[NC];
    int32_t i0, i1, j0, j1;
    uint32_t index;
};
template <class T, int NC> LH_HD SampleAdj<T, NC> sample_adj(const Bilinear<T>& s, int c0) {
    SampleAdj<T, NC> r;
    r.a = s.a;
    r.b = s.b;
    r.size_u = s.size_u;
    r.size_v = s.size_v;
    for (int c = 0; c < NC; c++) {
        const int ch = c0 + c;
        r.dda[c] = (T(1) - s.b) * (s.t10[ch] - s.t00[ch]) + s.b * (s.t11[ch] - s.t01[ch]);
        r.ddb[c] = (T(1) - s.a) * (s.t01[ch] - s.t00[ch]) + s.a * (s.t11[ch] - s.t10[ch]);
    }
    r.i0 = s.i0;
    r.i1 = s.i1;
    r.j0 = s.j0;
    r.j1 = s.j1;
    r.index = s.index;
    return r;
}

// Scalar fixed (non-differentiated) inputs of a pixel.
struct PixelScalars {
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

// Fixed inputs with the matrices held by value (the host checks).  Any type
// with the PixelScalars members and PV / NT / UVS (column, row) accessors
// stands in for it.
struct PixelFixed : PixelScalars {
    float pv[4][4];   // combined_perspective_view
    float nt[3][3];   // normal_transform, column major
    float uvs[4][4];  // uv_space_shadow_matrices[cascade] (cascade selected by the forward)
    LH_HD float PV(int c, int r) const { return pv[c][r]; }
    LH_HD float NT(int c, int r) const { return nt[c][r]; }
    LH_HD float UVS(int c, int r) const { return uvs[c][r]; }
};

// PV (v, w) and UVS (v, w), column-major, GLSL order.
template <class T, class F> LH_HD v3<T> xform_pv(const F& fx, v3<T> v, T w) {
    return {((T(fx.PV(0, 0)) * v.x + T(fx.PV(1, 0)) * v.y) + T(fx.PV(2, 0)) * v.z) + T(fx.PV(3, 0)) * w,
            ((T(fx.PV(0, 1)) * v.x + T(fx.PV(1, 1)) * v.y) + T(fx.PV(2, 1)) * v.z) + T(fx.PV(3, 1)) * w,
            ((T(fx.PV(0, 2)) * v.x + T(fx.PV(1, 2)) * v.y) + T(fx.PV(2, 2)) * v.z) + T(fx.PV(3, 2)) * w};
}
template <class T, class F> LH_HD T xform_pv_w(const F& fx, v3<T> v, T w) {
    return ((T(fx.PV(0, 3)) * v.x + T(fx.PV(1, 3)) * v.y) + T(fx.PV(2, 3)) * v.z) + T(fx.PV(3, 3)) * w;
}
template <class T, class F> LH_HD v3<T> xform_uvs(const F& fx, v3<T> v, T w) {
    return {((T(fx.UVS(0, 0)) * v.x + T(fx.UVS(1, 0)) * v.y) + T(fx.UVS(2, 0)) * v.z) + T(fx.UVS(3, 0)) * w,
            ((T(fx.UVS(0, 1)) * v.x + T(fx.UVS(1, 1)) * v.y) + T(fx.UVS(2, 1)) * v.z) + T(fx.UVS(3, 1)) * w,
            ((T(fx.UVS(0, 2)) * v.x + T(fx.UVS(1, 2)) * v.y) + T(fx.UVS(2, 2)) * v.z) + T(fx.UVS(3, 2)) * w};
}
template <class T, class F> LH_HD T xform_uvs_w(const F& fx, v3<T> v, T w) {
    return ((T(fx.UVS(0, 3)) * v.x + T(fx.UVS(1, 3)) * v.y) + T(fx.UVS(2, 3)) * v.z) + T(fx.UVS(3, 3)) * w;
}

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

// Compare results of one PCF tap (4 bits: texels 00, 10, 01, 11); the
// sampler's shadow_cmp(layer, i, j, ref) is 1 when ref < stored.
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
    const T inv_pi = T(1) / PI;
    T f90 = T(0.5) + T(2) * a * LoH * LoH;
    T ql = pow5(T(1) - NoL), qv = pow5(T(1) - NoV);
    T light = T(1) + (f90 - T(1)) * ql;
    T view = T(1) + (f90 - T(1)) * qv;
    BurleyOut<T> r;
    r.value = light * view * inv_pi;
    T dl_dNoL = -(f90 - T(1)) * T(5) * pow4(T(1) - NoL);
    T dv_dNoV = -(f90 - T(1)) * T(5) * pow4(T(1) - NoV);
    T dval_df90 = (ql * view + light * qv) * inv_pi;
    r.dNoL = dl_dNoL * view * inv_pi;
    r.dNoV = light * dv_dNoV * inv_pi;
    r.dLoH = dval_df90 * T(4) * a * LoH;
    r.da = dval_df90 * T(2) * LoH * LoH;
    return r;
}

// The world position the forward interpolates (CalcFullBary's lambda and
// InterpolateWithDeriv), in the IEEE arithmetic of the inputs given: it
// selects the cascade and places the PCF taps.
template <class T, class F> LH_HD v3<T> forward_world(const F& fx, const PixelParams<T>& p) {
    v3<T> C[3];
    T iw[3];
    v2<T> n[3];
    for (int k = 0; k < 3; k++) {
        C[k] = xform_pv(fx, p.W[k], T(1));
        iw[k] = T(1) / xform_pv_w(fx, p.W[k], T(1));
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
    return {(p.W[0].x * lam[0] + p.W[1].x * lam[1]) + p.W[2].x * lam[2],
            (p.W[0].y * lam[0] + p.W[1].y * lam[1]) + p.W[2].y * lam[2],
            (p.W[0].z * lam[0] + p.W[1].z * lam[1]) + p.W[2].z * lam[2]};
}

// The forward's discrete decisions at its world position (face flip,
// far-plane test, the 36 compare results of fx.cascade's layer).
template <class T, class F, class Sampler>
LH_HD void decide_at(F& fx, const PixelParams<T>& p, v3<T> world, const Sampler& smp) {
    v3<T> V = normalize(sub(v3<T>{T(fx.cam[0]), T(fx.cam[1]), T(fx.cam[2])}, world));
    v3<T> gn = cross(sub(p.W[1], p.W[0]), sub(p.W[2], p.W[0]));
    fx.flip = dot(gn, V) < T(0) ? -1.0f : 1.0f;
    v3<T> sc = xform_uvs(fx, world, T(1));
    T scw = xform_uvs_w(fx, world, T(1));
    if (scw != T(1)) sc = {sc.x / scw, sc.y / scw, sc.z / scw};  // x / 1 = x
    fx.shadow_const = sc.z > T(1) ? 1u : 0u;
    const uint32_t layer = fx.cascade > 3 ? 3u : fx.cascade;
    const T S = T(fx.shadow_size), ref = sc.z - T(fx.bias);
    // The taps' texel columns / rows: when consecutive (one texel apart, a
    // 1024-texel cascade) the 4 x 4 texels they share are compared once and
    // the 36 results picked from them; otherwise tap by tap.
    int32_t ix[3], iy[3];
    for (int k = 0; k < 3; k++) {
        T uu = (sc.x + T(k - 1) / T(1024)) * S - T(0.5), vv = (sc.y + T(k - 1) / T(1024)) * S - T(0.5);
        if (!(tabs(uu) < T(1e9))) uu = T(0);
        if (!(tabs(vv) < T(1e9))) vv = T(0);
        ix[k] = (int32_t)tfloor(uu);
        iy[k] = (int32_t)tfloor(vv);
    }
    if (ix[1] == ix[0] + 1 && ix[2] == ix[1] + 1 && iy[1] == iy[0] + 1 && iy[2] == iy[1] + 1) {
        uint32_t win = 0;  // bit 4 * row + column of the window at (ix[0], iy[0])
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++)
                win |= (smp.shadow_cmp(layer, ix[0] + c, iy[0] + r, ref) != T(0) ? 1u : 0u) << (4 * r + c);
        uint64_t bits = 0;
        for (int ox = 0; ox < 3; ox++)
            for (int oy = 0; oy < 3; oy++) {
                const uint32_t q = win >> (4 * oy + ox);
                bits |= (uint64_t)((q & 3u) | ((q >> 2) & 12u)) << (4 * (ox * 3 + oy));
            }
        fx.cmp = bits;
        return;
    }
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

template <class T, class F, class Sampler> LH_HD void decide(F& fx, const PixelParams<T>& p, const Sampler& smp) {
    decide_at(fx, p, forward_world(fx, p), smp);
}

// Forward geometry of a pixel in two parts: CalcFullBary's lambda and its
// intermediates (the screen derivatives only feed the normal map, which is
// not differentiated), then the interpolated world position / uv / normal
// and the view vector.
template <class T> struct Bary {
    v3<T> C[3];
    T iw[3];
    v2<T> ca, cb;
    T invDet;
    T dxr[3], dyr[3], ddx0[3], ddy0[3];
    T sx, sy;
    v2<T> dv;
    T wi;
    T av[3], lam[3];
};

template <class T> struct Interp {
    v3<T> world;
    v2<T> uv;
    v3<T> vd, V;
    v3<T> nk[3];
    v3<T> nt, n0, normal;
};

template <class T, class F> LH_HD void bary(const F& fx, const PixelParams<T>& p, Bary<T>& B) {
    v2<T> n[3];
    for (int k = 0; k < 3; k++) {
        B.C[k] = xform_pv(fx, p.W[k], T(1));
        B.iw[k] = fdiv(T(1), xform_pv_w(fx, p.W[k], T(1)));
        n[k] = {B.C[k].x * B.iw[k], B.C[k].y * B.iw[k]};
    }
    B.ca = {n[2].x - n[1].x, n[2].y - n[1].y};
    B.cb = {n[0].x - n[1].x, n[0].y - n[1].y};
    B.invDet = fdiv(T(1), B.ca.x * B.cb.y - B.cb.x * B.ca.y);
    B.dxr[0] = n[1].y - n[2].y;
    B.dxr[1] = n[2].y - n[0].y;
    B.dxr[2] = n[0].y - n[1].y;
    B.dyr[0] = n[2].x - n[1].x;
    B.dyr[1] = n[0].x - n[2].x;
    B.dyr[2] = n[1].x - n[0].x;
    for (int k = 0; k < 3; k++) {
        B.ddx0[k] = B.dxr[k] * B.invDet * B.iw[k];
        B.ddy0[k] = B.dyr[k] * B.invDet * B.iw[k];
    }
    B.sx = (B.ddx0[0] * T(1) + B.ddx0[1] * T(1)) + B.ddx0[2] * T(1);
    B.sy = (B.ddy0[0] * T(1) + B.ddy0[1] * T(1)) + B.ddy0[2] * T(1);
    B.dv = {T(fx.ndc[0]) - n[0].x, T(fx.ndc[1]) - n[0].y};
    B.wi = fdiv(T(1), (B.iw[0] + B.dv.x * B.sx) + B.dv.y * B.sy);
    B.av[0] = (B.iw[0] + B.dv.x * B.ddx0[0]) + B.dv.y * B.ddy0[0];
    B.av[1] = (T(0) + B.dv.x * B.ddx0[1]) + B.dv.y * B.ddy0[1];
    B.av[2] = (T(0) + B.dv.x * B.ddx0[2]) + B.dv.y * B.ddy0[2];
    for (int k = 0; k < 3; k++) B.lam[k] = B.wi * B.av[k];
}

template <class T, class F>
LH_HD void interp(const F& fx, const PixelParams<T>& p, const T lam[3], Interp<T>& I) {
    // InterpolateWithDeriv value: dot(v, lambda)
    I.world = {(p.W[0].x * lam[0] + p.W[1].x * lam[1]) + p.W[2].x * lam[2],
               (p.W[0].y * lam[0] + p.W[1].y * lam[1]) + p.W[2].y * lam[2],
               (p.W[0].z * lam[0] + p.W[1].z * lam[1]) + p.W[2].z * lam[2]};
    v2<T> uvs[3];
    for (int k = 0; k < 3; k++) uvs[k] = {p.UV[k].x * T(fx.ts[0]), p.UV[k].y * T(fx.ts[1])};
    I.uv = {((uvs[0].x * lam[0] + uvs[1].x * lam[1]) + uvs[2].x * lam[2]) + T(fx.toff[0]),
            ((uvs[0].y * lam[0] + uvs[1].y * lam[1]) + uvs[2].y * lam[2]) + T(fx.toff[1])};
    I.vd = sub(v3<T>{T(fx.cam[0]), T(fx.cam[1]), T(fx.cam[2])}, I.world);
    I.V = fnormalize(I.vd);
    for (int k = 0; k < 3; k++) I.nk[k] = fnormalize(p.N[k]);
    const v3<T> ni = {(I.nk[0].x * lam[0] + I.nk[1].x * lam[1]) + I.nk[2].x * lam[2],
                      (I.nk[0].y * lam[0] + I.nk[1].y * lam[1]) + I.nk[2].y * lam[2],
                      (I.nk[0].z * lam[0] + I.nk[1].z * lam[1]) + I.nk[2].z * lam[2]};
    I.nt = {(T(fx.NT(0, 0)) * ni.x + T(fx.NT(1, 0)) * ni.y) + T(fx.NT(2, 0)) * ni.z,
            (T(fx.NT(0, 1)) * ni.x + T(fx.NT(1, 1)) * ni.y) + T(fx.NT(2, 1)) * ni.z,
            (T(fx.NT(0, 2)) * ni.x + T(fx.NT(1, 2)) * ni.y) + T(fx.NT(2, 2)) * ni.z};
    I.n0 = fnormalize(I.nt);
    I.normal = mul(I.n0, T(fx.flip));
}

// PCF shadow with the cascade and the compare results fixed; the weights
// stay differentiable in the shadow coordinate.
template <class T> struct ShadowTerm {
    T value, dx, dy;  // value and d/d(sc.xy)
    T scx, scy, inv_w;
};

template <class T, class F> LH_HD ShadowTerm<T> shadow_term(const F& fx, v3<T> world) {
    v3<T> sc = xform_uvs(fx, world, T(1));
    const T inv_w = fdiv(T(1), xform_uvs_w(fx, world, T(1)));
    sc = {sc.x * inv_w, sc.y * inv_w, sc.z * inv_w};
    T shadow = T(0), dsx = T(0), dsy = T(0);
    const T S = T(fx.shadow_size);
    // with every compare 0 each tap's value and derivatives are exactly 0
    if (fx.cmp != 0) {
        for (int ox = -1; ox <= 1; ox++)
            for (int oy = -1; oy <= 1; oy++) {
                T da, db;
                const uint32_t tap = (uint32_t)((ox + 1) * 3 + (oy + 1));
                shadow += pcf_tap((uint32_t)(fx.cmp >> (4 * tap)) & 15u, sc.x + T(ox) / T(1024),
                                  sc.y + T(oy) / T(1024), S, da, db);
                dsx += da * S;
                dsy += db * S;
            }
    }
    const T ninth = T(1) / T(9);
    ShadowTerm<T> r;
    r.value = fx.shadow_const ? T(1) : shadow * ninth;
    r.dx = dsx * ninth;
    r.dy = dsy * ninth;
    r.scx = sc.x;
    r.scy = sc.y;
    r.inv_w = inv_w;
    return r;
}

// What the surface reverse hands to the geometry reverse.
template <class T> struct SurfaceGrad {
    v3<T> normal, V;
    v2<T> uv;
    T shadow;
};

// Materials, SH ambient and BRDF (pbr.glsl:44-96) of a surface point:
// writes the radiance to *out and, when g is non-null, runs the reverse for
// `gout`: the light, base-colour-factor and texel gradients go to *g, the
// gradients of the surface inputs to *sg.
template <class T, class F, class Sampler>
LH_HD void surface(const F& fx, const PixelParams<T>& p, const Sampler& smp, v2<T> uv, v3<T> normal, v3<T> V,
                   T shadow, v3<T>* out, v3<T> gout, PixelGrad<T>* g, SurfaceGrad<T>* sg) {
    const T PI = T(3.14159265358979323846f);
    // materials: keep only what the reverse needs of the two samples
    SampleAdj<T, 3> sb;
    SampleAdj<T, 2> sm;
    v3<T> texc;
    T rough, metal;
    {
        const Bilinear<T> b = smp.sample(fx.base_tex, uv);
        texc = {bilerp(b, 0), bilerp(b, 1), bilerp(b, 2)};
        sb = sample_adj<T, 3>(b, 0);
    }
    {
        const Bilinear<T> m = smp.sample(fx.mr_tex, uv);
        rough = bilerp(m, 1);
        metal = bilerp(m, 2);
        sm = sample_adj<T, 2>(m, 1);
    }
    v3<T> base = mulv(texc, p.bcf);
    // (a normal map would replace `normal` here; not differentiated)
    // SH ambient: only sh[0] = sh[2] = 0.025 are non-zero
    const T amb_level = T(0.025f);
    T amb = amb_level + amb_level * normal.y;
    v3<T> diffuse = mul(base, T(1) - metal);
    v3<T> ambient = mul(diffuse, amb);
    // BRDF (pbr.glsl:44-96)
    v3<T> L = p.sun;
    v3<T> h0 = add(V, L);
    v3<T> H = fnormalize(h0);
    T refl = (T(1.5) - T(1)) / (T(1.5) + T(1));
    refl = refl * refl;
    v3<T> f0 = add(mul(v3<T>{refl, refl, refl}, T(1) - metal), mul(base, metal));
    T NoVr = dot(normal, V), NoLr = dot(normal, L), NoHr = dot(normal, H), LoHr = dot(L, H);
    T NoV = tclamp(NoVr, T(1e-5f), T(1)), NoL = tclamp(NoLr, T(0), T(1));
    T NoH = tclamp(NoHr, T(0), T(1)), LoH = tclamp(LoHr, T(0), T(1));
    T a = rough * rough;
    T a2 = a * a;
    T fq = (NoH * a2 - NoH) * NoH + T(1);
    T D = fdiv(a2, PI * fq * fq);
    T q5 = pow5(T(1) - LoH);
    v3<T> Fr{f0.x + (T(1) - f0.x) * q5, f0.y + (T(1) - f0.y) * q5, f0.z + (T(1) - f0.z) * q5};
    T sL = fsqrt((-NoL * a2 + NoL) * NoL + a2), sV = fsqrt((-NoV * a2 + NoV) * NoV + a2);
    T GGXL = NoV * sL, GGXV = NoL * sV;
    T Vis = fdiv(T(0.5), GGXV + GGXL);
    BurleyOut<T> fb = burley(NoV, NoL, LoH, a);
    v3<T> pre{(diffuse.x * fb.value + Fr.x * (D * Vis)) * NoL, (diffuse.y * fb.value + Fr.y * (D * Vis)) * NoL,
              (diffuse.z * fb.value + Fr.z * (D * Vis)) * NoL};
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
    // sun = irr * (pi * shadow) * light
    v3<T> g_irr{gout.x * sun_scale * light.x, gout.y * sun_scale * light.y, gout.z * sun_scale * light.z};
    g->light = {gout.x * irr.x * sun_scale, gout.y * irr.y * sun_scale, gout.z * irr.z * sun_scale};
    sg->shadow = PI * ((gout.x * irr.x * light.x + gout.y * irr.y * light.y) + gout.z * irr.z * light.z);
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
    T g_DV = ((g_pre.x * Fr.x + g_pre.y * Fr.y) + g_pre.z * Fr.z) * NoL;
    T g_NoL = (g_pre.x * (diffuse.x * fb.value + Fr.x * DV) + g_pre.y * (diffuse.y * fb.value + Fr.y * DV)) +
              g_pre.z * (diffuse.z * fb.value + Fr.z * DV);
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
    T g_den = fdiv(-g_Vis * T(0.5), den * den);
    T g_GGXV = g_den, g_GGXL = g_den;
    // GGXL = NoV * sL, sL = sqrt(NoL^2 (1 - a2) + a2)
    g_NoV += g_GGXL * sL;
    T g_sL = g_GGXL * NoV;
    g_NoL += g_GGXV * sV;
    T g_sV = g_GGXV * NoL;
    T g_a2 = T(0);
    // sL^2 = (-NoL a2 + NoL) NoL + a2
    const T hL = fdiv(g_sL, T(2) * sL), hV = fdiv(g_sV, T(2) * sV);
    g_NoL += hL * (T(2) * NoL * (T(1) - a2));
    g_a2 += hL * (T(1) - NoL * NoL);
    g_NoV += hV * (T(2) * NoV * (T(1) - a2));
    g_a2 += hV * (T(1) - NoV * NoV);
    // D = a2 / (pi fq^2), fq = NoH^2 (a2 - 1) + 1
    T g_fq = fdiv(-g_D * T(2) * a2, PI * fq * fq * fq);
    g_a2 += fdiv(g_D, PI * fq * fq) + g_fq * NoH * NoH;
    g_NoH += g_fq * T(2) * NoH * (a2 - T(1));
    // F_c = f0_c + (1 - f0_c) q5, q5 = (1 - LoH)^5
    v3<T> g_f0{g_F.x * (T(1) - q5), g_F.y * (T(1) - q5), g_F.z * (T(1) - q5)};
    T g_q5 = (g_F.x * (T(1) - f0.x) + g_F.y * (T(1) - f0.y)) + g_F.z * (T(1) - f0.z);
    g_LoH += -g_q5 * T(5) * pow4(T(1) - LoH);
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
    v3<T> g_h0 = fnormalize_adj(h0, H, g_H);
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
            g_uv.x += gt[c] * sb.dda[c] * sb.size_u;
            g_uv.y += gt[c] * sb.ddb[c] * sb.size_v;
        }
        T wm[4] = {(T(1) - sm.a) * (T(1) - sm.b), sm.a * (T(1) - sm.b), (T(1) - sm.a) * sm.b, sm.a * sm.b};
        T gm[2] = {g_rough, g_metal};
        for (int c = 0; c < 2; c++) {
            for (int q = 0; q < 4; q++) g->mr_texel[q][c] = gm[c] * wm[q];
            g_uv.x += gm[c] * sm.dda[c] * sm.size_u;
            g_uv.y += gm[c] * sm.ddb[c] * sm.size_v;
        }
    }
    sg->normal = g_normal;
    sg->V = g_V;
    sg->uv = g_uv;
}

// Opaque copies of the vertex attributes: a recomputation from them is not
// merged with an earlier one by the device compiler.
template <class T> LH_HD PixelParams<T> opaque_params(PixelParams<T> p) {
    for (int k = 0; k < 3; k++) {
        opaque(p.W[k].x), opaque(p.W[k].y), opaque(p.W[k].z);
        opaque(p.N[k].x), opaque(p.N[k].y), opaque(p.N[k].z);
        opaque(p.UV[k].x), opaque(p.UV[k].y);
    }
    return p;
}

// Reverse of the geometry: from the gradients of the surface inputs (and of
// the world position through the shadow term) to the vertex attributes.
// The forward geometry is recomputed here in two steps -- the lambdas and
// interpolants for the first half of the reverse, the barycentric
// intermediates again for the second -- so that only a few values are live
// at any point.
template <class T, class F>
LH_HD void geometry_adjoint(const F& fx, const PixelParams<T>& p0, const SurfaceGrad<T>& sg, v3<T> g_world,
                            PixelGrad<T>* g) {
    T lam[3], g_lam[3];
    {
        const PixelParams<T> p = opaque_params(p0);
        {
            Bary<T> B;
            bary(fx, p, B);
            lam[0] = B.lam[0];
            lam[1] = B.lam[1];
            lam[2] = B.lam[2];
        }
        Interp<T> I;
        interp(fx, p, lam, I);
        // normal = flip * normalize(nt); nt = NT ni; ni = sum lam_k nk; nk = normalize(N_k)
        v3<T> g_n0 = mul(sg.normal, T(fx.flip));
        v3<T> g_nt = fnormalize_adj(I.nt, I.n0, g_n0);
        v3<T> g_ni{(T(fx.NT(0, 0)) * g_nt.x + T(fx.NT(0, 1)) * g_nt.y) + T(fx.NT(0, 2)) * g_nt.z,
                   (T(fx.NT(1, 0)) * g_nt.x + T(fx.NT(1, 1)) * g_nt.y) + T(fx.NT(1, 2)) * g_nt.z,
                   (T(fx.NT(2, 0)) * g_nt.x + T(fx.NT(2, 1)) * g_nt.y) + T(fx.NT(2, 2)) * g_nt.z};
        for (int k = 0; k < 3; k++) {
            g->N[k] = fnormalize_adj(p.N[k], I.nk[k], mul(g_ni, lam[k]));
            g_lam[k] = dot(I.nk[k], g_ni);
        }
        // V = normalize(cam - world)
        g_world = sub(g_world, fnormalize_adj(I.vd, I.V, sg.V));
        // uv = sum lam_k uvs_k + offset, uvs_k = UV_k * scale
        for (int k = 0; k < 3; k++) {
            g->UV[k] = {sg.uv.x * lam[k] * T(fx.ts[0]), sg.uv.y * lam[k] * T(fx.ts[1])};
            g_lam[k] += sg.uv.x * (p.UV[k].x * T(fx.ts[0])) + sg.uv.y * (p.UV[k].y * T(fx.ts[1]));
        }
        // world = sum lam_k W_k.  The lambdas sum to 1 for every input, so
        // their gradients may be shifted by a common term: W_k - W_0 instead
        // of W_k keeps float32 from cancelling world-scale coordinates.
        for (int k = 0; k < 3; k++) {
            g->W[k] = mul(g_world, lam[k]);
            g_lam[k] += dot(sub(p.W[k], p.W[0]), g_world);
        }
    }
    Bary<T> G;
    bary(fx, opaque_params(p0), G);
    // ---- barycentrics: lam_k = wi * av_k
    const T wi = G.wi;
    T g_wi = (g_lam[0] * G.av[0] + g_lam[1] * G.av[1]) + g_lam[2] * G.av[2];
    T g_av[3] = {g_lam[0] * wi, g_lam[1] * wi, g_lam[2] * wi};
    T g_iiw = -g_wi * wi * wi;
    T g_iw[3] = {T(0), T(0), T(0)};
    T g_ddx0[3] = {T(0), T(0), T(0)}, g_ddy0[3] = {T(0), T(0), T(0)};
    v2<T> g_dv{T(0), T(0)};
    g_iw[0] += g_iiw;
    g_dv.x += g_iiw * G.sx;
    g_dv.y += g_iiw * G.sy;
    T g_sx = g_iiw * G.dv.x, g_sy = g_iiw * G.dv.y;
    g_iw[0] += g_av[0];
    for (int k = 0; k < 3; k++) {
        g_dv.x += g_av[k] * G.ddx0[k];
        g_dv.y += g_av[k] * G.ddy0[k];
        g_ddx0[k] += g_av[k] * G.dv.x + g_sx;
        g_ddy0[k] += g_av[k] * G.dv.y + g_sy;
    }
    T g_invDet = T(0), g_dxr[3], g_dyr[3];
    for (int k = 0; k < 3; k++) {
        g_dxr[k] = g_ddx0[k] * G.invDet * G.iw[k];
        g_dyr[k] = g_ddy0[k] * G.invDet * G.iw[k];
        g_invDet += g_ddx0[k] * G.dxr[k] * G.iw[k] + g_ddy0[k] * G.dyr[k] * G.iw[k];
        g_iw[k] += g_ddx0[k] * G.dxr[k] * G.invDet + g_ddy0[k] * G.dyr[k] * G.invDet;
    }
    v2<T> g_n[3] = {{-g_dv.x, -g_dv.y}, {T(0), T(0)}, {T(0), T(0)}};
    T g_det = -g_invDet * G.invDet * G.invDet;
    v2<T> g_ca{g_det * G.cb.y, -g_det * G.cb.x}, g_cb{-g_det * G.ca.y, g_det * G.ca.x};
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
        T gCx = g_n[k].x * G.iw[k], gCy = g_n[k].y * G.iw[k];
        g_iw[k] += g_n[k].x * G.C[k].x + g_n[k].y * G.C[k].y;
        T gCw = -g_iw[k] * G.iw[k] * G.iw[k];
        // C = PV (W, 1): dW_j = sum_r PV[j][r] dC_r  (C.z carries no gradient)
        g->W[k].x += (T(fx.PV(0, 0)) * gCx + T(fx.PV(0, 1)) * gCy) + T(fx.PV(0, 3)) * gCw;
        g->W[k].y += (T(fx.PV(1, 0)) * gCx + T(fx.PV(1, 1)) * gCy) + T(fx.PV(1, 3)) * gCw;
        g->W[k].z += (T(fx.PV(2, 0)) * gCx + T(fx.PV(2, 1)) * gCy) + T(fx.PV(2, 3)) * gCw;
    }
}

// The two halves of shade(): shade_surface() runs the forward and the
// reverse of everything but the geometry (filling g's light, light
// direction, base-colour-factor and texel gradients), shade_geometry() the
// geometry reverse (g's vertex gradients).  What passes between them:
template <class T> struct SurfaceState {
    ShadowTerm<T> sh;
    SurfaceGrad<T> sg;
};

template <class T, class F, class Sampler>
LH_HD void shade_surface(const F& fx, const PixelParams<T>& p, const Sampler& smp, v3<T>* out, v3<T> gout,
                         PixelGrad<T>* g, SurfaceState<T>* st) {
    Bary<T> B;
    bary(fx, p, B);
    Interp<T> I;
    interp(fx, p, B.lam, I);
    st->sh = shadow_term(fx, I.world);
    surface(fx, p, smp, I.uv, I.normal, I.V, st->sh.value, out, gout, g, &st->sg);
    if (g) g->differentiated = fx.has_normal_map == 0;
}

template <class T, class F>
LH_HD void shade_geometry(const F& fx, const PixelParams<T>& p, const SurfaceState<T>& st, PixelGrad<T>* g) {
    // shadow: d/d(sc.xy) through the PCF weights, compare results fixed;
    // sc.xy = (UVS (world,1)).xy / w with w = row 3 (constant 1 for the
    // orthographic cascades)
    v3<T> g_world{T(0), T(0), T(0)};
    if (!fx.shadow_const) {
        T gsx = st.sg.shadow * st.sh.dx, gsy = st.sg.shadow * st.sh.dy;
        T gw = -(gsx * st.sh.scx + gsy * st.sh.scy) * st.sh.inv_w;
        gsx *= st.sh.inv_w;
        gsy *= st.sh.inv_w;
        g_world.x = (T(fx.UVS(0, 0)) * gsx + T(fx.UVS(0, 1)) * gsy) + T(fx.UVS(0, 3)) * gw;
        g_world.y = (T(fx.UVS(1, 0)) * gsx + T(fx.UVS(1, 1)) * gsy) + T(fx.UVS(1, 3)) * gw;
        g_world.z = (T(fx.UVS(2, 0)) * gsx + T(fx.UVS(2, 1)) * gsy) + T(fx.UVS(2, 3)) * gw;
    }
    geometry_adjoint(fx, p, st.sg, g_world, g);
}

// Forward (into *out) and, when `g` is non-null, the reverse pass for the
// upstream gradient `gout` of the pixel's RGB, with the discrete decisions
// in `fx` (decide()) held fixed.  The geometry may be given relative to any
// origin (PV, UVS and fx.cam expressed for the same origin): the backward
// kernel uses the camera, which keeps float32 from cancelling world-scale
// coordinates.  `smp` provides sample(tex, uv) -> Bilinear.
template <class T, class F, class Sampler>
LH_HD void shade(const F& fx, const PixelParams<T>& p, const Sampler& smp, v3<T>* out, v3<T> gout, PixelGrad<T>* g) {
    SurfaceState<T> st;
    shade_surface(fx, p, smp, out, gout, g, &st);
    if (g) shade_geometry(fx, p, st, g);
}

}  // namespace shade
}  // namespace lh
