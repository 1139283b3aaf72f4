// Host check of lbmg::div_rn (divrn.cuh), compiled from the kernel's own header: the quotient of
// the reciprocal-pair division against IEEE x / y, bit for bit, for the divisors the FP64 step
// uses (the speed-of-sound constants, tau over its whole range, densities near 1 and across the
// supported range [2^-30, 2^30]) and dividends that make the quotient fall next to a rounding
// midpoint (the hardest cases for a correction step), at random magnitudes, and special values.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "divrn.cuh"
#include "lattice.cuh"

using namespace lbmg;

static uint64_t bits(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
}

static long long check_divisor(double y, std::mt19937_64& rng, long long n)
{
    const DivRN d = make_div_rn(y, 1.0 / y);
    std::uniform_real_distribution<double> mant(1.0, 2.0);
    std::uniform_int_distribution<int> expo(-905, 905), small(-60, 10), pick(0, 3);
    long long wrong = 0;
    auto test = [&](double x) {
        const double a = div_rn(x, d), b = x / y;
        if (bits(a) != bits(b) && !(std::isnan(a) && std::isnan(b))) {
            if (wrong < 5) std::printf("  y %a x %a: %a vs %a\n", y, x, a, b);
            ++wrong;
        }
    };
    for (long long k = 0; k < n; ++k) {
        const int e = pick(rng) == 0 ? expo(rng) : small(rng);
        const double sign = (rng() & 1) ? -1.0 : 1.0;
        switch (k % 3) {
        case 0:  // random dividend
            test(sign * std::ldexp(mant(rng), e));
            break;
        default: {
            // a quotient next to the midpoint between m and its successor: x = RN(mid * y) and
            // its neighbours
            const double m = std::ldexp(mant(rng), e);
            const double mid = m + (std::nextafter(m, 2 * m) - m) / 2;
            double x = sign * (mid * y);
            for (int s = 0; s < 3; ++s) x = std::nextafter(x, 0.0);
            for (int s = 0; s < 7; ++s, x = std::nextafter(x, sign * INFINITY)) test(x);
        }
        }
    }
    const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 0x1p-1074, -0x1p-1030, 0x1p-900,
                               0x1.fffffffffffffp-901, 0x1p+900, 0x1.0000000000001p+900, 1.0, -1.0, y, -y};
    for (double x : specials) test(x);
    return wrong;
}

int main()
{
    std::mt19937_64 rng(20261204);
    std::vector<double> ys = {kCS2, kCS4x2, kCS2x2};
    for (double omega : {1.0, 1.7, 1.8, 1.9, 1.95, 0.6, 1.5}) ys.push_back(1.0 / omega);
    for (double tau : {0.5000001, 0.51, 0.6, 0.75, 1.0, 1.25, 1.9999999}) ys.push_back(tau);
    std::uniform_real_distribution<double> near1(0.9, 1.1), wide(-30.0, 29.0);
    for (int k = 0; k < 20; ++k) ys.push_back(near1(rng));
    for (int k = 0; k < 10; ++k) ys.push_back(std::ldexp(1.0 + near1(rng) / 2, static_cast<int>(wide(rng))));
    ys.push_back(0x1p-30);
    ys.push_back(0x1.fffffffffffffp+29);
    long long wrong = 0, total = 0;
    for (double y : ys) {
        const long long n = 300000;
        wrong += check_divisor(y, rng, n);
        total += n;
    }
    // the lattice constants' reciprocal pairs
    const struct { double y, zh, zl; } tab[] = {
        {kCS2, cs2_div().zh, cs2_div().zl}, {kCS4x2, cs4x2_div().zh, cs4x2_div().zl}, {kCS2x2, cs2x2_div().zh, cs2x2_div().zl}};
    for (const auto& t : tab) {
        if (t.zh != 1.0 / t.y || std::fabs(t.zl - std::fma(-t.y, t.zh, 1.0) / t.y) > 0x1p-100) {
            std::printf("  constant pair of %a is not RN(1/y), (1 - y zh)/y\n", t.y);
            ++wrong;
        }
    }
    std::printf("divisors %zu, dividend cases %lld: %lld wrong\n", ys.size(), total, wrong);
    return wrong == 0 ? 0 : 1;
}
