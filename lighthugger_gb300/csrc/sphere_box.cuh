// Whether a meshlet can reach a pixel centre of a view, from its world
// sphere alone (before any vertex is loaded).
//
// The meshlet cull writes the raster's draw record with the meshlet's world
// sphere, which holds every vertex position the raster computes (the radius
// carries the rounding of the vertices' transform).  This bounds the
// sphere's axis-aligned box through the view matrix in clip space, widened
// by a bound on the float rounding of both that bound and the raster's own
// transform of any point of the box; divides the clip interval of x (and y)
// by the one of w (all w of the box above 0; x / w is monotone in each, so
// the extremes lie at the interval corners); takes it to pixels, widened by
// the rounding of the divide, the viewport transform and the 1/256-pixel
// snap.  When that screen box holds no pixel centre of the view, no
// triangle of the meshlet (clipped or not: clipping only cuts triangles
// down) covers one, and the raster skips the meshlet.  Undecided (a box
// corner at or behind the camera plane, or non-finite values): not skipped.
// Host-compilable for the CPU check in tests/native.
#pragma once

#include <cmath>
#include <cstdint>

#include "lh/shared.h"

#if defined(__CUDACC__)
#define LH_SB_HD __host__ __device__ __forceinline__
#else
#define LH_SB_HD inline
#endif

namespace lh {

LH_SB_HD float sb_min(float a, float b) { return a < b ? a : b; }
LH_SB_HD float sb_max(float a, float b) { return a > b ? a : b; }

// Rounding allowance, relative to the sum of the absolute terms of a
// transform: the raster's 4-term sums with separately rounded products are
// within 4 units in the last place (2^-22) of it, this bound's own within as
// much again; 2^-20 leaves a factor two.
constexpr float kSbRel = 1.0f / 1048576.0f;

// Interval [lo, hi] of row `r` (0: x, 1: y, 3: w) of vp applied to the box
// (c ± R), widened by the rounding allowance.
LH_SB_HD void sb_row(const lh_mat4& vp, int r, float cx, float cy, float cz, float R, float& lo, float& hi) {
    auto el = [&](int col) {
        const lh_vec4& v = vp.cols[col];
        return r == 0 ? v.x : (r == 1 ? v.y : v.w);
    };
    const float m0 = el(0), m1 = el(1), m2 = el(2), m3 = el(3);
    const float mid = ((m0 * cx + m1 * cy) + m2 * cz) + m3;
    const float ext = (std::fabs(m0) + std::fabs(m1) + std::fabs(m2)) * R;
    const float terms = ((std::fabs(m0) * (std::fabs(cx) + R) + std::fabs(m1) * (std::fabs(cy) + R)) +
                         std::fabs(m2) * (std::fabs(cz) + R)) + std::fabs(m3);
    const float wid = ext + terms * kSbRel + ext * kSbRel;
    lo = mid - wid;
    hi = mid + wid;
}

// Pixel-centre columns (or rows) i of [0, n) with i + 0.5 in the screen
// interval of ndc [a, b] (half extent h = n / 2), widened: empty -> true.
LH_SB_HD bool sb_no_centre(float a, float b, float h, uint32_t n) {
    float lo = a * h + h, hi = b * h + h;
    const float m = 1.0f / 128.0f + (std::fabs(lo) + std::fabs(hi) + h) * kSbRel;
    lo -= m;
    hi += m;
    if (!(lo <= hi)) return false;                      // NaN: undecided
    if (hi < 0.5f || lo > (float)n - 0.5f) return true;  // entirely off the view's centres
    // first and last centre index inside, within [0, n - 1]
    const float fl = std::ceil(lo - 0.5f), fh = std::floor(hi - 0.5f);
    return fl > fh;
}

LH_SB_HD bool sphere_misses_centres(const lh_mat4& vp, float cx, float cy, float cz, float R, uint32_t W, uint32_t H) {
    if (!(R >= 0.0f) || !(std::fabs(cx) + std::fabs(cy) + std::fabs(cz) + R < 1e30f)) return false;
    float xl, xh, yl, yh, wl, wh;
    sb_row(vp, 3, cx, cy, cz, R, wl, wh);
    if (!(wl > 1e-6f) || !(wh < 1e30f)) return false;
    sb_row(vp, 0, cx, cy, cz, R, xl, xh);
    sb_row(vp, 1, cx, cy, cz, R, yl, yh);
    // x / w over the box: the extremes at the corners of [xl, xh] x [wl, wh]
    const float ax = sb_min(xl / wl, xl / wh), bx = sb_max(xh / wl, xh / wh);
    const float ay = sb_min(yl / wl, yl / wh), by = sb_max(yh / wl, yh / wh);
    // the divide's rounding, relative to the quotients
    const float dx = (std::fabs(ax) + std::fabs(bx)) * kSbRel, dy = (std::fabs(ay) + std::fabs(by)) * kSbRel;
    return sb_no_centre(ax - dx, bx + dx, (float)W * 0.5f, W) || sb_no_centre(ay - dy, by + dy, (float)H * 0.5f, H);
}

}  // namespace lh
