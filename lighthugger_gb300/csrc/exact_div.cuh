// Correctly rounded quotient x / n of small non-negative integers held as
// floats (pixel column / image width), or of any float 0 <= x <= 9 by n = 9
// (the PCF's sum over its nine taps), without a division per call: from the
// correctly rounded reciprocal r = 1 / n (one IEEE division, computed once),
// q0 = x * r, the remainder x - n * q0 (exact in one fused multiply-add) and
// q0 + remainder * r rounded once -- the correction step of P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990.  The host check
// tests/native/exact_div_check.cpp compares it bit for bit with the IEEE
// quotient for every integer pair 0 <= x <= n <= 16384 and for every float
// 0 <= x <= 9 (subnormals included) with n = 9.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define LH_ED_HD __host__ __device__ __forceinline__
#else
#define LH_ED_HD inline
#endif

namespace lh {

constexpr int kExactDivMaxCount = 16384;  // the largest n the host check covers

LH_ED_HD float fma_rn(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// x / n for integers 0 <= x <= n <= kExactDivMaxCount, or for n = 9 and any
// float 0 <= x <= 9; rcp_n = 1.0f / n.
LH_ED_HD float div_by_count(float x, float n, float rcp_n) {
    const float q0 = x * rcp_n;
    const float rem = fma_rn(-n, q0, x);
    return fma_rn(rem, rcp_n, q0);
}

}  // namespace lh
