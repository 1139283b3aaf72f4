// Host check of lbmg::bgk_adjoint (adjoint.cuh), compiled from the kernel's own source: J^T lam
// for the BGK map against the transpose of a central-difference Jacobian of that map, in FP64,
// for D3Q15 / D3Q19 / D3Q27, FP64 and FP32 instantiations, at random states near equilibrium.
#include <cmath>
#include <cstdio>
#include <random>

#include "adjoint.cuh"

using namespace lbmg;

// g -> g + omega (feq(g) - g), feq_q = w_q rho (1 + A cu + B cu^2 - C uu)
template <class L>
static void bgk(const double* g, double omega, double* out)
{
    using K = AdjConst<double>;
    double rho = 0, jx = 0, jy = 0, jz = 0;
    for (int q = 0; q < L::Q; ++q) {
        rho += g[q];
        jx += g[q] * L::c(q, 0);
        jy += g[q] * L::c(q, 1);
        jz += g[q] * L::c(q, 2);
    }
    const double ux = jx / rho, uy = jy / rho, uz = jz / rho, uu = ux * ux + uy * uy + uz * uz;
    for (int q = 0; q < L::Q; ++q) {
        const double cu = L::c(q, 0) * ux + L::c(q, 1) * uy + L::c(q, 2) * uz;
        const double feq = L::w(q) * rho * (1 + K::A * cu + K::B * cu * cu - K::C * uu);
        out[q] = g[q] + omega * (feq - g[q]);
    }
}

template <class L, class T>
static double check(std::mt19937_64& rng, double omega)
{
    constexpr int Q = L::Q;
    std::normal_distribution<double> n01(0.0, 1.0);
    double g[Q], lam0[Q];
    const double drift[3] = {0.04 * n01(rng), 0.04 * n01(rng), 0.04 * n01(rng)};
    for (int q = 0; q < Q; ++q) {
        const double cu = L::c(q, 0) * drift[0] + L::c(q, 1) * drift[1] + L::c(q, 2) * drift[2];
        g[q] = L::w(q) * (1.0 + 3.0 * cu + 0.02 * n01(rng));
        lam0[q] = n01(rng);
    }
    // want_p = sum_q lam_q dBGK_q/dg_p
    const double h = 1e-6;
    double want[Q], gp[Q], gm[Q], fp[Q], fm[Q];
    for (int p = 0; p < Q; ++p) {
        for (int q = 0; q < Q; ++q) gp[q] = gm[q] = g[q];
        gp[p] += h;
        gm[p] -= h;
        bgk<L>(gp, omega, fp);
        bgk<L>(gm, omega, fm);
        want[p] = 0;
        for (int q = 0; q < Q; ++q) want[p] += lam0[q] * (fp[q] - fm[q]) / (2 * h);
    }
    double rho = 0, jx = 0, jy = 0, jz = 0;
    for (int q = 0; q < Q; ++q) {
        rho += g[q];
        jx += g[q] * L::c(q, 0);
        jy += g[q] * L::c(q, 1);
        jz += g[q] * L::c(q, 2);
    }
    T lam[Q];
    for (int q = 0; q < Q; ++q) lam[q] = static_cast<T>(lam0[q]);
    bgk_adjoint<L, T>(lam, T(rho), T(jx), T(jy), T(jz), T(omega));
    double err = 0, scale = 0;
    for (int p = 0; p < Q; ++p) {
        err = std::fmax(err, std::fabs(static_cast<double>(lam[p]) - want[p]));
        scale = std::fmax(scale, std::fabs(want[p]));
    }
    return err / scale;
}

template <class L>
static bool run(std::mt19937_64& rng)
{
    double e64 = 0, e32 = 0;
    for (int k = 0; k < 200; ++k) {
        const double omega = 0.6 + 1.35 * (k % 10) / 9.0;  // 0.6 .. 1.95
        e64 = std::fmax(e64, check<L, double>(rng, omega));
        e32 = std::fmax(e32, check<L, float>(rng, omega));
    }
    const bool ok = e64 < 1e-7 && e32 < 1e-5;
    std::printf("D3Q%d max rel err fp64 %.3e fp32 %.3e %s\n", L::Q, e64, e32, ok ? "ok" : "FAIL");
    return ok;
}

int main()
{
    std::mt19937_64 rng(11);
    bool ok = run<Lattice<15>>(rng);
    ok = run<Lattice<19>>(rng) && ok;
    ok = run<Lattice<27>>(rng) && ok;
    return ok ? 0 : 1;
}
