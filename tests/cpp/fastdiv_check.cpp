// Host check of lbmg::make_fastdiv (domain.cuh): n / d == (umulhi(n, m) + n) >> l for divisors and
// numerators across the 32-bit range, with umulhi written out as the device instruction computes it.
#include <cstdint>
#include <cstdio>
#include <random>

#include "domain.cuh"

int main()
{
    std::mt19937_64 rng(7);
    uint64_t bad = 0, checked = 0;
    auto check = [&](uint32_t n, uint32_t d) {
        const lbmg::FastDiv f = lbmg::make_fastdiv(d);
        const uint32_t hi = static_cast<uint32_t>((static_cast<uint64_t>(n) * f.m) >> 32);
        const uint32_t q = static_cast<uint32_t>((static_cast<uint64_t>(hi) + n) >> f.l);
        bad += q != n / d;
        ++checked;
    };
    for (uint32_t d = 1; d < 5000; ++d)
        for (uint32_t n : {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 0x7fffffffu, 0xffffffffu}) check(n, d);
    for (int k = 0; k < 2000000; ++k)
        check(static_cast<uint32_t>(rng()), static_cast<uint32_t>(rng() % 0xfffffffeull) + 1u);
    std::printf("%llu checked, %llu wrong\n", (unsigned long long)checked, (unsigned long long)bad);
    return bad != 0;
}
