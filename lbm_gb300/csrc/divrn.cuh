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
// [2^-30, 2^30] (positive), and x outside [2^-900, 2^900] in magnitude (subnormals, infinities and
// NaN included) takes the plain division, so that the quotient stays inside [2^-930, 2^930] and
// the remainder above 2^-1012. A zero x returns x itself (+-0 / y = +-0 for y > 0) on the fast
// path: a flow at rest divides zeros everywhere. The host check tests/cpp/div_rn_check.cpp
// compares div_rn with IEEE division on midpoint-adjacent and random quotients.
#pragma once

#include <cmath>
#include <cuda_runtime.h>

namespace lbmg {

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

__host__ __device__ __forceinline__ double div_rn(double x, const DivRN& d)
{
    const double ax = fabs(x);
    if (ax <= 0x1p+900 && (ax >= 0x1p-900 || ax == 0.0)) {
        const double q0 = fma(x, d.zh, x * d.zl);
        const double q = fma(fma(-q0, d.y, x), d.zh, q0);
        return ax == 0.0 ? x : q;
    }
    return x / d.y;
}

}  // namespace lbmg
