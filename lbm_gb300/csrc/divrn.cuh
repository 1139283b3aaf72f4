// Correctly rounded FP64 division by a divisor known in advance.
//
// The FP64 step reproduces the reference's arithmetic bit for bit, and the reference divides: by
// tau (collision.hpp:68), by C_S*C_S, 2*C_S^4 and 2*C_S^2 (collision.hpp:45-46) and by the
// density (collision.hpp:29). An IEEE division is a sequence of about ten FP64 instructions on the
// GPU, and FP64 issues at a small fraction of the FP32 rate on this GPU. With the divisor y fixed
// in advance, x / y rounded to nearest takes four:
//   - zh = RN(1/y) and zl ~ (1 - y zh) / y, precomputed (the residual 1 - y zh is exact in one fma
//     when zh is the correctly rounded reciprocal);
//   - q0 = RN(x zh + RN(x zl)) lies within half an ulp plus about 2^-100 relative of x / y
//     (Brisebarre, Muller and Raina, "Accelerating correctly rounded floating-point division when
//     the divisor is known in advance", IEEE Trans. Computers 53(8), 2004), so it is a faithful
//     quotient;
//   - with a faithful quotient q0 and the correctly rounded reciprocal zh, the remainder
//     r = x - y q0 is exact in one fma and RN(q0 + r zh) is RN(x / y) (P. Markstein, "Computation
//     of elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
//     1990; the theorem that completes IA-64 division).
// The theorems assume no underflow or overflow in the intermediate steps: callers keep y inside
// [2^-30, 2^30] (positive), and x outside [2^-900, 2^900) in magnitude (subnormals, infinities and
// NaN included) takes the plain division, so that the quotient stays inside [2^-930, 2^930] and
// the remainder above 2^-1012. A zero x returns x itself (+-0 / y = +-0 for y > 0) on the fast
// path: a flow at rest divides zeros everywhere. The host check tests/cpp/div_rn_check.cpp
// compares div_rn with IEEE division on midpoint-adjacent and random quotients.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace lbmg {

// The upper and lower 32 bits of x (the upper word holds the sign, the exponent and the top of
// the significand).
__host__ __device__ __forceinline__ void words(double x, uint32_t& hi, uint32_t& lo)
{
#ifdef __CUDA_ARCH__
    hi = static_cast<uint32_t>(__double2hiint(x));
    lo = static_cast<uint32_t>(__double2loint(x));
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    hi = static_cast<uint32_t>(b >> 32);
    lo = static_cast<uint32_t>(b);
#endif
}

struct DivRN {
    double y;   // the divisor
    double zh;  // RN(1 / y)
    double zl;  // (1 - y zh) / y, to about 2^-50 relative
};

// From the divisor and its correctly rounded reciprocal (1.0 / y on the host, __drcp_rn(y) on the
// device).
__host__ __device__ inline DivRN make_div_rn(double y, double zh)
{
    DivRN d;
    d.y = y;
    d.zh = zh;
    d.zl = fma(-y, zh, 1.0) * zh;
    return d;
}

// The range tests work on the exponent bits with integer instructions: FP64 comparisons would
// occupy the FP64 pipe, whose time this division saves.
__host__ __device__ __forceinline__ double div_rn(double x, const DivRN& d)
{
    uint32_t hi, lo;
    words(x, hi, lo);
    const uint32_t e = hi & 0x7fffffffu;  // |x| without the sign
    const bool in_range = e - 0x07b00000u < 0x78300000u - 0x07b00000u;  // 2^-900 <= |x| < 2^900
    if (in_range || (e | lo) == 0u) {
        const double q0 = fma(x, d.zh, x * d.zl);
        const double q = fma(fma(-q0, d.y, x), d.zh, q0);
        return in_range ? q : x;
    }
    return x / d.y;
}

}  // namespace lbmg
