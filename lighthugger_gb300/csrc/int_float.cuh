// Integer -> float conversions for the rasteriser's edge functions.
//
// Two edge functions are converted per covered fragment.  Small values (the
// common case: fragments of small triangles) go through the significand of
// 1.5 * 2^23 -- one integer add and one float subtract -- instead of a
// conversion instruction.  Every routine returns exactly what the
// round-to-nearest-even conversion returns (__int2float_rn / __ll2float_rn,
// static_cast<float> on the host), so depths stay bit exact.  i64_to_f32_rn
// is the integer-only 64-bit conversion; host-compilable for the CPU check in
// tests/native.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define LH_IF_HD __host__ __device__ __forceinline__
#else
#define LH_IF_HD inline
#endif

namespace lh {

LH_IF_HD float bits_to_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, 4);
    return f;
#endif
}

LH_IF_HD int clz64(uint64_t a) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)a);
#else
    return __builtin_clzll(a);
#endif
}

// Round-to-nearest-even conversion of a signed 64-bit integer.
LH_IF_HD float i64_to_f32_rn(int64_t v) {
    const uint32_t sign = v < 0 ? 0x80000000u : 0u;
    const uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
    if (a == 0) return 0.0f;
    int e = 63 - clz64(a);  // position of the leading one
    uint64_t q;
    if (e <= 23) {
        q = a << (23 - e);
    } else {
        const int sh = e - 23;
        q = a >> sh;
        const uint64_t rem = a & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull))) q++;
        if (q >> 24) {
            q >>= 1;
            e++;
        }
    }
    return bits_to_float(sign | ((uint32_t)(e + 127) << 23) | ((uint32_t)q & 0x7FFFFFu));
}

// Round-to-nearest-even conversion of 0 <= v < 2^46 with FP32 adds only:
// v = a * 2^23 + b with a, b < 2^23; each part is an exact float (placed in
// the significand of 2^46, resp. 2^23, and that power subtracted), so the
// one rounding of their sum is the rounding of v.
LH_IF_HD float u46_to_f32_rn(uint64_t v) {
    const float fa = bits_to_float(0x56800000u | (uint32_t)(v >> 23)) - 70368744177664.0f;
    const float fb = bits_to_float(0x4B000000u | ((uint32_t)v & 0x7FFFFFu)) - 8388608.0f;
    return fa + fb;
}

// The same for any unsigned 32-bit v (its high part v >> 23 has 9 bits).
LH_IF_HD float u32_to_f32_rn(uint32_t v) {
    const float fa = bits_to_float(0x56800000u | (v >> 23)) - 70368744177664.0f;
    const float fb = bits_to_float(0x4B000000u | (v & 0x7FFFFFu)) - 8388608.0f;
    return fa + fb;
}

// Round-to-nearest-even conversion of a signed 32-bit integer: values below
// 2^22 in magnitude are placed in the significand of 1.5 * 2^23 (exact: one
// integer add and one float subtract), the rest take the general routine.
LH_IF_HD float i32_to_f32_rn(int32_t v) {
    if (v > -(1 << 22) && v < (1 << 22)) return bits_to_float(0x4B400000u + (uint32_t)v) - 12582912.0f;
#if defined(__CUDA_ARCH__)
    return __int2float_rn(v);
#else
    return i64_to_f32_rn((int64_t)v);
#endif
}

}  // namespace lh
