// Runs of covered pixels along a row, for the big-triangle chunks.
//
// Along one pixel row of a chunk the rasteriser's integer edge function is
// E(k) = e0 + k * dx at the chunk's k-th pixel (e0 its value at the first,
// dx = 256 * (the edge's y extent)), and the pixel passes the edge's test
// when E(k) >= bias (bias 0 or 1: the top-left rule).  E is affine in k, so
// the passing k form one run; a triangle's covered pixels in the row are
// the intersection of its three edges' runs.  clip_run narrows [lo, hi] to
// one edge's run.  The step count at the run's end is a quotient, estimated
// in float and corrected by one exact integer step each way: for chunks of
// at most 256 pixels the estimate's error stays far below one step, so the
// run holds exactly the pixels the per-pixel test passes.  Host-compilable
// for the CPU check in tests/native.
#pragma once

#include <cmath>
#include <cstdint>

#include "int_float.cuh"

#if defined(__CUDACC__)
#define LH_ER_HD __host__ __device__ __forceinline__
#else
#define LH_ER_HD inline
#endif

namespace lh {

// |v| as float, near enough for the estimate (exact below 2^46; above, the
// low 18 bits are dropped).  FP32 and integer adds only.
LH_ER_HD float abs_to_f32(int64_t v) {
    const uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
    const bool big = (a >> 46) != 0;
    return u46_to_f32_rn(big ? a >> 18 : a) * (big ? 262144.0f : 1.0f);
}

// 1 / x, near enough for the estimate (a few ulps).
LH_ER_HD float approx_rcp(float x) {
#if defined(__CUDA_ARCH__)
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}

LH_ER_HD int32_t f32_ceil_to_i32(float x) {
#if defined(__CUDA_ARCH__)
    return __float2int_ru(x);
#else
    return (int32_t)std::ceil(x);
#endif
}
LH_ER_HD int32_t f32_floor_to_i32(float x) {
#if defined(__CUDA_ARCH__)
    return __float2int_rd(x);
#else
    return (int32_t)std::floor(x);
#endif
}

// The reciprocal of an edge's step dx = 256 * dy (dy: the edge's y extent
// in 1/256 pixels), shared by every row of the triangle's chunks (0 for dy = 0).
LH_ER_HD float run_inv_step(int32_t dy) { return dy == 0 ? 0.0f : approx_rcp(std::fabs((float)dy) * 256.0f); }

// Narrow [lo, hi] (pixels 0 .. n-1 of the row, n <= 256) to the pixels where
// e0 + k * dx >= bias; an empty result has lo > hi.  inv = run_inv_step(dy).
LH_ER_HD void clip_run(int64_t e0, int64_t dx, int64_t bias, int32_t n, float inv, int32_t& lo, int32_t& hi) {
    if (dx == 0) {
        if (e0 < bias) hi = -1;
        return;
    }
    if (dx > 0) {
        // first passing pixel: ceil((bias - e0) / dx)
        const int64_t need = bias - e0;
        if (need <= 0) return;
        if (need > (int64_t)(n - 1) * dx) {
            hi = -1;
            return;
        }
        int32_t k = f32_ceil_to_i32(abs_to_f32(need) * inv);
        k = k < 1 ? 1 : (k > n - 1 ? n - 1 : k);
        if (e0 + (int64_t)(k - 1) * dx >= bias) k--;
        else if (e0 + (int64_t)k * dx < bias) k++;
        if (k > lo) lo = k;
    } else {
        // last passing pixel: floor((e0 - bias) / -dx)
        const int64_t room = e0 - bias;
        if (room < 0) {
            hi = -1;
            return;
        }
        if (room >= (int64_t)(n - 1) * -dx) return;
        int32_t k = f32_floor_to_i32(abs_to_f32(room) * inv);
        k = k < 0 ? 0 : (k > n - 2 ? n - 2 : k);
        if (e0 + (int64_t)(k + 1) * dx >= bias) k++;
        else if (e0 + (int64_t)k * dx < bias) k--;
        if (k < hi) hi = k;
    }
}

}  // namespace lh
