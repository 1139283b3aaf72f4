// Device kernels of the lattice Boltzmann step, templated on the lattice model L and the
// population storage type S. Each step_*.cu translation unit includes this file and
// instantiates it for one storage type (step_fp64.cu is compiled with -fmad=false so that the
// FP64 path performs every operation the reference performs, in the same order, unfused).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "domain.cuh"
#include "lattice.cuh"
#include "tma.cuh"

namespace lbmg {

// ------------------------------------------------------------------------------------------
// Storage policies. FP64 stores populations as they are and computes in FP64 exactly as the
// reference does. The other stores hold s_q = f_q - w_q and compute in FP32 on s directly, so
// the O(1) part of every population never enters the rounding.
// ------------------------------------------------------------------------------------------
template <class S>
struct Store;

template <>
struct Store<double> {
    using C = double;
    static constexpr bool kShifted = false;
    __device__ static __forceinline__ double ld(const double* p) { return *p; }
    __device__ static __forceinline__ void st(double* p, double v) { *p = v; }
    __device__ static __forceinline__ void st_stream(double* p, double v) { __stcs(p, v); }
};
template <>
struct Store<float> {
    using C = float;
    static constexpr bool kShifted = true;
    __device__ static __forceinline__ float ld(const float* p) { return *p; }
    __device__ static __forceinline__ void st(float* p, float v) { *p = v; }
    __device__ static __forceinline__ void st_stream(float* p, float v) { __stcs(p, v); }
};
template <>
struct Store<__half> {
    using C = float;
    static constexpr bool kShifted = true;
    __device__ static __forceinline__ float ld(const __half* p) { return __half2float(*p); }
    __device__ static __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
    __device__ static __forceinline__ void st_stream(__half* p, float v)
    {
        const unsigned short b = __half_as_ushort(__float2half_rn(v));
        asm volatile("st.global.cs.b16 [%0], %1;" ::"l"(p), "h"(b) : "memory");
    }
};
template <>
struct Store<__nv_bfloat16> {
    using C = float;
    static constexpr bool kShifted = true;
    __device__ static __forceinline__ float ld(const __nv_bfloat16* p)
    {
        return __bfloat162float(*p);
    }
    __device__ static __forceinline__ void st(__nv_bfloat16* p, float v)
    {
        *p = __float2bfloat16_rn(v);
    }
    __device__ static __forceinline__ void st_stream(__nv_bfloat16* p, float v)
    {
        const unsigned short b = __bfloat16_as_ushort(__float2bfloat16_rn(v));
        asm volatile("st.global.cs.b16 [%0], %1;" ::"l"(p), "h"(b) : "memory");
    }
};

// Storage value <-> FP64 population f_q.
template <class L, class S>
__device__ __forceinline__ double to_f64(typename Store<S>::C v, int q)
{
    if constexpr (Store<S>::kShifted)
        return L::w(q) + static_cast<double>(v);
    else
        return static_cast<double>(v);
}
template <class L, class S>
__device__ __forceinline__ typename Store<S>::C from_f64(double f, int q)
{
    if constexpr (Store<S>::kShifted)
        return static_cast<float>(f - L::w(q));
    else
        return f;
}

// ------------------------------------------------------------------------------------------
// Indexing.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int cidx(const Geom& g, int x, int y, int z)
{
    return kXOff + x + g.XS * (y + g.YS * z);
}

__device__ __forceinline__ int wrap_axis(int v, int l, bool per)
{
    if (per) {
        if (v < 1) v += l;
        else if (v > l) v -= l;
    }
    return v;
}

// Neighbour (x+dx, y+dy, z+dz) with periodic wrap; writes its coordinates.
__device__ __forceinline__ void nbr_xyz(const Geom& g, int x, int y, int z, int dx, int dy,
                                        int dz, int& nx, int& ny, int& nz)
{
    nx = wrap_axis(x + dx, g.xl, g.per & 1);
    ny = wrap_axis(y + dy, g.yl, g.per & 2);
    nz = wrap_axis(z + dz, g.zl, g.per & 4);
}

__device__ __forceinline__ bool interior(const Geom& g, int x, int y, int z)
{
    return x >= 1 && x <= g.xl && y >= 1 && y <= g.yl && z >= 1 && z <= g.zl;
}

// Reference cell order (domain.hpp:60-64) for host-facing arrays.
__device__ __forceinline__ size_t ref_idx(const Geom& g, int x, int y, int z)
{
    return static_cast<size_t>(x) +
           static_cast<size_t>(g.xl + 2) *
               (static_cast<size_t>(y) + static_cast<size_t>(g.yl + 2) * static_cast<size_t>(z));
}

__device__ __forceinline__ bool is_fluid(uint8_t f) { return f <= kFluidWall; }

// ------------------------------------------------------------------------------------------
// FP64 arithmetic in the reference's operation order (collision.hpp:6-70, boundary.hpp).
// Multiplications by a lattice velocity component c in {-1, 0, 1} are written as an add, a
// subtract or nothing: x*1 = x, x*(-1) = -x and x + (+-0) = x for the running sums here (they
// start at +0.0 and can never be -0.0), so the results are bit-identical.
// ------------------------------------------------------------------------------------------
template <class L>
__device__ __forceinline__ double density_exact(const double (&f)[L::Q])
{
    double rho = 0.0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) rho += f[q];
    return rho;
}

// Momentum sum_q f_q c_qd (d outer, q inner: collision.hpp:19-24), before the division.
template <class L>
__device__ __forceinline__ double momentum_exact(const double (&f)[L::Q], int d)
{
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        const int c = L::c(q, d);
        if (c > 0) s += f[q];
        else if (c < 0) s -= f[q];
    }
    return s;
}

// compute_feq (collision.hpp:33-51) for one direction q. Every division is the correctly
// rounded division of divrn.cuh, bit-identical to the reference's.
template <class L>
__device__ __forceinline__ double feq_exact(int q, double rho, double u0, double u1, double u2)
{
    double cu = 0.0;
    double uu = 0.0;
    const int c0 = rt_c<L>(q, 0), c1 = rt_c<L>(q, 1), c2 = rt_c<L>(q, 2);
    if (c0 > 0) cu += u0; else if (c0 < 0) cu -= u0;
    uu += u0 * u0;
    if (c1 > 0) cu += u1; else if (c1 < 0) cu -= u1;
    uu += u1 * u1;
    if (c2 > 0) cu += u2; else if (c2 < 0) cu -= u2;
    uu += u2 * u2;
    return rt_w<L>(q) * rho *
           (1 + div_rn(cu, cs2_div()) + div_rn((cu) * (cu), cs4x2_div()) - div_rn(uu, cs2x2_div()));
}

// The three velocity components m[1..3] / rho (collision.hpp:27-29), correctly rounded: through
// the reciprocal pair of rho where rho lies in div_rn's divisor range, by plain division otherwise
// (a diverged state).
__device__ __forceinline__ void velocity_exact(const double (&m)[4], double& u0, double& u1, double& u2)
{
    const double rho = m[0];
    uint32_t hi, lo;
    words(rho, hi, lo);
    if (hi - 0x3e100000u < 0x41d00000u - 0x3e100000u) {  // 2^-30 <= rho < 2^30 (integer test)
        const DivRN r = make_div_rn(rho, __drcp_rn(rho));
        u0 = div_rn(m[1], r);
        u1 = div_rn(m[2], r);
        u2 = div_rn(m[3], r);
    } else {
        u0 = m[1] / rho;
        u1 = m[2] / rho;
        u2 = m[3] / rho;
    }
}

// BGKCollision::collide (collision.hpp:60-70), operation for operation; tau is the relaxation
// time's reciprocal pair. Opposite directions q and inv q = Q-1-q share their equilibrium terms:
// c_{inv q}.u, summed in the reference's order, is exactly -(c_q.u) (or +0 where c_q.u is +0),
// so cu/cs2 only changes sign (1 + a absorbs the sign of a zero) and cu^2/(2 cs4) is the same.
// The equilibria are those of compute_feq bit for bit, with half the divisions.
template <class L>
__device__ __forceinline__ void collide_exact(double (&f)[L::Q], const DivRN& tau, double (&m)[4])
{
    const double rho = density_exact<L>(f);
    m[0] = rho;
    m[1] = momentum_exact<L>(f, 0);
    m[2] = momentum_exact<L>(f, 1);
    m[3] = momentum_exact<L>(f, 2);
    double u0, u1, u2;
    velocity_exact(m, u0, u1, u2);
    double uu = 0.0;
    uu += u0 * u0;
    uu += u1 * u1;
    uu += u2 * u2;
    const double c = div_rn(uu, cs2x2_div());
#pragma unroll
    for (int q = 0; q < L::REST; ++q) {
        const int qb = L::Q - 1 - q;
        double cu = 0.0;
        if (L::c(q, 0) > 0) cu += u0; else if (L::c(q, 0) < 0) cu -= u0;
        if (L::c(q, 1) > 0) cu += u1; else if (L::c(q, 1) < 0) cu -= u1;
        if (L::c(q, 2) > 0) cu += u2; else if (L::c(q, 2) < 0) cu -= u2;
        const double a = div_rn(cu, cs2_div());
        const double b = div_rn((cu) * (cu), cs4x2_div());
        const double wr = L::w(q) * rho;
        const double feq = wr * (1 + a + b - c);
        const double feqb = wr * (1 - a + b - c);
        f[q] -= div_rn(f[q] - feq, tau);
        f[qb] -= div_rn(f[qb] - feqb, tau);
    }
    constexpr int R = L::REST;
    const double feq = L::w(R) * rho * (1 + 0.0 + 0.0 - c);
    f[R] -= div_rn(f[R] - feq, tau);
}

// Momentum sum_q f_q c_qd of populations kept in memory at fs[q * stride].
template <class L, class T>
__device__ __forceinline__ T momentum_mem(const T* fs, int stride, int d)
{
    T s = 0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        const int c = L::c(q, d);
        if (c > 0) s += fs[q * stride];
        else if (c < 0) s -= fs[q * stride];
    }
    return s;
}

// Value a boundary cell's handler writes into its direction q = inv(p) for the fluid cell that
// sees it in direction p, from that fluid cell's post-collision populations fs[k * stride]
// (boundary.hpp:14-214). rho_s = density of fs. p may be known only at run time.
template <class L>
__device__ __forceinline__ double bc_value_exact(const BcEntry& b, int p, const double* fs, int stride,
                                                 double rho_s, const double* vcell)
{
    const int q = inv<L>(p);
    switch (b.type) {
    case kMovingWall: {  // boundary.hpp:52-66
        double cu = 0.0;
        const int c0 = rt_c<L>(q, 0), c1 = rt_c<L>(q, 1), c2 = rt_c<L>(q, 2);
        if (c0 > 0) cu += b.v[0]; else if (c0 < 0) cu -= b.v[0];
        if (c1 > 0) cu += b.v[1]; else if (c1 < 0) cu -= b.v[1];
        if (c2 > 0) cu += b.v[2]; else if (c2 < 0) cu -= b.v[2];
        const double finv = fs[p * stride];
        return finv + div_rn(2.0 * rt_w<L>(q) * rho_s * cu, cs2_div());
    }
    case kInflow: {  // boundary.hpp:173-179
        const double* v = vcell ? vcell : b.v;
        return feq_exact<L>(q, b.rho, v[0], v[1], v[2]);
    }
    case kOutflow:     // boundary.hpp:137-148
    case kPressure: {  // boundary.hpp:203-212
        const double u0 = momentum_mem<L>(fs, stride, 0) / b.rho;
        const double u1 = momentum_mem<L>(fs, stride, 1) / b.rho;
        const double u2 = momentum_mem<L>(fs, stride, 2) / b.rho;
        return feq_exact<L>(q, b.rho, u0, u1, u2) + feq_exact<L>(p, b.rho, u0, u1, u2) - fs[p * stride];
    }
    default:  // kNoSlip, boundary.hpp:22-29
        return fs[p * stride];
    }
}

// ------------------------------------------------------------------------------------------
// FP32 arithmetic on shifted populations s_q = f_q - w_q. With rho = 1 + drho,
//   f_eq,q - w_q = w_q (drho + rho (cu/cs2 + cu^2/(2 cs4) - uu/(2 cs2)))
// keeps the reference's truncated speed of sound (collision.hpp:45-46).
// ------------------------------------------------------------------------------------------
constexpr float kA = static_cast<float>(1.0 / kCS2);
constexpr float kB = static_cast<float>(1.0 / kCS4x2);
constexpr float kC = static_cast<float>(1.0 / kCS2x2);

template <class L>
__device__ __forceinline__ float seq_shifted(int q, float drho, float rho, float ux, float uy,
                                             float uz, float uu_c)
{
    const float cu = rt_c<L>(q, 0) * ux + rt_c<L>(q, 1) * uy + rt_c<L>(q, 2) * uz;
    return static_cast<float>(rt_w<L>(q)) * (drho + rho * (cu * (kA + cu * kB) - uu_c));
}

// Mass and momentum over opposite pairs: the sum s_q + s_inv(q) enters the mass, the difference
// s_q - s_inv(q) each momentum component where c_q has one (one subtraction per pair instead of
// one per direction and component).
template <class L>
__device__ __forceinline__ void moments_shifted(const float (&s)[L::Q], float& drho, float& jx,
                                                float& jy, float& jz)
{
    drho = s[L::REST]; jx = 0.f; jy = 0.f; jz = 0.f;
#pragma unroll
    for (int q = 0; q < L::REST; ++q) {
        const int qb = L::Q - 1 - q;
        const float sum = s[q] + s[qb], dif = s[q] - s[qb];
        drho += sum;
        if (L::c(q, 0) > 0) jx += dif; else if (L::c(q, 0) < 0) jx -= dif;
        if (L::c(q, 1) > 0) jy += dif; else if (L::c(q, 1) < 0) jy -= dif;
        if (L::c(q, 2) > 0) jz += dif; else if (L::c(q, 2) < 0) jz -= dif;
    }
}

// The per-cell quantities of the shifted BGK relaxation, from the moments.
struct ShiftedEq {
    float ux, uy, uz, base, rA, rB;
};
__device__ __forceinline__ ShiftedEq shifted_eq(float drho, float jx, float jy, float jz)
{
    ShiftedEq e;
    const float rho = 1.f + drho;
    // the hardware reciprocal (rcp.approx: at most 1 ulp from 1/rho, rho near 1): the velocity
    // keeps FP32 rounding level, for one instruction instead of a correctly rounded sequence
    float ir;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ir) : "f"(rho));
    e.ux = jx * ir, e.uy = jy * ir, e.uz = jz * ir;
    e.base = fmaf(-rho * kC, e.ux * e.ux + e.uy * e.uy + e.uz * e.uz, drho);
    e.rA = rho * kA, e.rB = rho * kB;
    return e;
}
// The rest population relaxed.
template <class L>
__device__ __forceinline__ float relax_rest(const ShiftedEq& e, float omega, float s)
{
    return fmaf(omega, fmaf(static_cast<float>(L::w(L::REST)), e.base, -s), s);
}
// The pair (q, inv q) relaxed in one packed FP32x2 FMA chain: each lane performs the operations
// fmaf(omega, fmaf(w, sym +- asym, -s), s) exactly as written for one population.
template <class L>
__device__ __forceinline__ float2 relax_pair(const ShiftedEq& e, int q, float omega, float sq, float sqb)
{
    const float cu = L::c(q, 0) * e.ux + L::c(q, 1) * e.uy + L::c(q, 2) * e.uz;
    const float sym = fmaf(cu * cu, e.rB, e.base);
    const float asym = cu * e.rA;
    const float w = static_cast<float>(L::w(q));
    const float2 ev = make_float2(sym + asym, sym - asym);
    const float2 sv = make_float2(sq, sqb);
    const float2 t = __ffma2_rn(make_float2(w, w), ev, make_float2(-sv.x, -sv.y));
    return __ffma2_rn(make_float2(omega, omega), t, sv);
}

// BGK on shifted populations. Per opposite pair (q, inv q) the equilibria share
// sym = drho - rho uu/(2 cs2) + rho cu^2/(2 cs4) and differ in the sign of asym = rho cu/cs2:
//   s_eq,q - ... = w_q (sym +- asym),   s_q <- s_q + omega (w_q (sym +- asym) - s_q).
template <class L>
__device__ __forceinline__ void collide_shifted(float (&s)[L::Q], float omega, float (&m)[4])
{
    float drho, jx, jy, jz;
    moments_shifted<L>(s, drho, jx, jy, jz);
    m[0] = drho;
    m[1] = jx;
    m[2] = jy;
    m[3] = jz;
    const ShiftedEq e = shifted_eq(drho, jx, jy, jz);
    constexpr int R = L::REST;
    s[R] = relax_rest<L>(e, omega, s[R]);
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const int qb = L::Q - 1 - q;
        const float2 r = relax_pair<L>(e, q, omega, s[q], s[qb]);
        s[q] = r.x;
        s[qb] = r.y;
    }
}

// FP32 counterpart of bc_value_exact on shifted populations ss[k * stride]; drho_s and j are the
// post-collision moments of the fluid cell.
template <class L>
__device__ __forceinline__ float bc_value_shifted(const BcEntry& b, int p, const float* ss, int stride,
                                                  float drho_s, float jx, float jy, float jz,
                                                  const double* vcell)
{
    const int q = inv<L>(p);
    switch (b.type) {
    case kMovingWall: {
        const float rho = 1.f + drho_s;
        const float cu = rt_c<L>(q, 0) * static_cast<float>(b.v[0]) +
                         rt_c<L>(q, 1) * static_cast<float>(b.v[1]) +
                         rt_c<L>(q, 2) * static_cast<float>(b.v[2]);
        return ss[p * stride] + 2.f * static_cast<float>(rt_w<L>(q)) * rho * cu * kA;
    }
    case kInflow: {
        const double* v = vcell ? vcell : b.v;
        const float r = static_cast<float>(b.rho);
        const float ux = static_cast<float>(v[0]), uy = static_cast<float>(v[1]),
                    uz = static_cast<float>(v[2]);
        return seq_shifted<L>(q, r - 1.f, r, ux, uy, uz, (ux * ux + uy * uy + uz * uz) * kC);
    }
    case kOutflow:
    case kPressure: {
        const float r = static_cast<float>(b.rho);
        const float ir = 1.f / r;
        const float ux = jx * ir, uy = jy * ir, uz = jz * ir;
        const float uu_c = (ux * ux + uy * uy + uz * uz) * kC;
        return seq_shifted<L>(q, r - 1.f, r, ux, uy, uz, uu_c) +
               seq_shifted<L>(p, r - 1.f, r, ux, uy, uz, uu_c) - ss[p * stride];
    }
    default:
        return ss[p * stride];
    }
}

// ------------------------------------------------------------------------------------------
// The fused time step: pull-stream + BGK collide + boundary handlers, in place (AA pattern).
// ODD = the step number (1-based) is odd: populations are pulled from the neighbours and pushed
// to them; even steps read and write the cell's own slots. Every cell's read set equals its
// write set, so cells are independent within a step and may be updated in any order.
// ------------------------------------------------------------------------------------------
template <class S>
struct StepParams {
    S* pop;
    const uint8_t* flag;
    const uint2* link;     // per fluid cell: x bit q = the pull neighbour x - c_q is not fluid;
                           // y = LinkRecord row or kNoRecord
    const BcEntry* bc;
    const double* profile;
    const int* edge;       // layout indices of the kFluidEdge cells, increasing
    int n_edge;
    const LinkRecord* ltab;
    const uint8_t* wmask;  // per row segment: bit w = warp w covers kFluidBulk cells only
    int* err;              // set to 1 when a bounded wait gives up
    double* mon;           // kMonBuckets x 4 FP64 accumulators of the step's mass and momentum,
                           // or nullptr
    double* mon_prev;      // the previous monitored step's accumulators, which block 0 adds up into
    double* mon_prev_out;  // mon_prev_out[0..3] and clears; or nullptr
    typename Store<S>::C* rec;  // per cell (layout index i): rec[4i..4i+3] = mass and momentum of
                                // the populations the cell pulled this step, or nullptr; 16-byte
                                // aligned (one vector store per cell)
    Geom g;
    DivRN tau;             // relaxation time and its reciprocal pair (FP64 storage)
    float omega;
};

// Collides f in place; m receives the mass and momentum of the populations it started from, in
// the compute type (shifted storage: the mass minus 1, so that nothing here needs FP64, whose
// rate on this GPU is a small fraction of FP32's; the monitor converts inside its own branch).
template <class L, class S>
__device__ __forceinline__ void collide_any(typename Store<S>::C (&f)[L::Q], const StepParams<S>& P,
                                            typename Store<S>::C (&m)[4])
{
    if constexpr (Store<S>::kShifted)
        collide_shifted<L>(f, P.omega, m);
    else
        collide_exact<L>(f, P.tau, m);
}

// The four record values of one cell, as whole vectors (one 16-byte access for FP32, two for
// FP64): four scalar accesses 16 bytes apart would each touch four times the sectors they use.
__device__ __forceinline__ void st_rec4(float* r, float a, float b, float c, float d)
{
    __stcs(reinterpret_cast<float4*>(r), make_float4(a, b, c, d));
}
__device__ __forceinline__ void st_rec4(double* r, double a, double b, double c, double d)
{
    __stcs(reinterpret_cast<double2*>(r), make_double2(a, b));
    __stcs(reinterpret_cast<double2*>(r) + 1, make_double2(c, d));
}
__device__ __forceinline__ void ld_rec4(const float* r, float& a, float& b, float& c, float& d)
{
    const float4 v = __ldcs(reinterpret_cast<const float4*>(r));
    a = v.x, b = v.y, c = v.z, d = v.w;
}
__device__ __forceinline__ void ld_rec4(const double* r, double& a, double& b, double& c, double& d)
{
    const double2 u = __ldcs(reinterpret_cast<const double2*>(r));
    const double2 v = __ldcs(reinterpret_cast<const double2*>(r) + 1);
    a = u.x, b = u.y, c = v.x, d = v.y;
}

// Stores a cell's pre-collision mass and momentum for the adjoint's recompute segments.
template <class S>
__device__ __forceinline__ void record_moments(typename Store<S>::C* rec, int i, const typename Store<S>::C (&m)[4])
{
    using T = typename Store<S>::C;
    st_rec4(rec + 4 * static_cast<size_t>(i), Store<S>::kShifted ? T(1) + m[0] : m[0], m[1], m[2], m[3]);
}

// Handler values of an edge cell: for every direction p toward a non-fluid neighbour m (bit
// inv(p) of `link`), the value m's handler writes for this cell, stored where this cell pulls
// direction inv(p) next step: after an odd step plane inv(p) at the cell, after an even step
// plane p at m. fs[k * stride] holds the cell's post-collision populations. Ghost-fluid and
// free-slip neighbours are skipped: their side passes fill those slots.
template <class L, class S, bool ODD>
__device__ __forceinline__ void store_handler_values(const StepParams<S>& P, int x, int y, int z, int i,
                                                     uint32_t link, const typename Store<S>::C* fs,
                                                     int stride)
{
    using St = Store<S>;
    using T = typename St::C;
    T m0, m1, m2, m3;  // post-collision moments for the handlers that need them
    if constexpr (St::kShifted) {
        m0 = 0.f;
#pragma unroll
        for (int q = 0; q < L::Q; ++q) m0 += fs[q * stride];
        m1 = momentum_mem<L>(fs, stride, 0);
        m2 = momentum_mem<L>(fs, stride, 1);
        m3 = momentum_mem<L>(fs, stride, 2);
    } else {
        m0 = 0.0;
#pragma unroll
        for (int q = 0; q < L::Q; ++q) m0 += fs[q * stride];
        m1 = m2 = m3 = 0.0;
    }
    uint32_t bits = link & ((1u << L::Q) - 1u);
    while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1u;
        const int p = inv<L>(b);
        int mx, my, mz;
        nbr_xyz(P.g, x, y, z, rt_c<L>(p, 0), rt_c<L>(p, 1), rt_c<L>(p, 2), mx, my, mz);
        const uint8_t flm = P.flag[cidx(P.g, mx, my, mz)];
        if (flm < kFirstHandler) continue;
        const BcEntry& be = P.bc[flm - kFirstHandler];
        if (be.type == kFreeSlip) continue;
        const double* vcell = nullptr;
        if (be.type == kInflow && be.has_profile) vcell = P.profile + 3 * ref_idx(P.g, mx, my, mz);
        T val;
        if constexpr (St::kShifted)
            val = bc_value_shifted<L>(be, p, fs, stride, m0, m1, m2, m3, vcell);
        else
            val = bc_value_exact<L>(be, p, fs, stride, m0, vcell);
        if (ODD)
            St::st(P.pop + static_cast<size_t>(b) * P.g.PS + i, val);
        else
            St::st(P.pop + static_cast<size_t>(p) * P.g.PS + cidx(P.g, mx, my, mz), val);
    }
}

// Post-collision stores of an edge cell: the plain AA stores, wrapping on periodic axes.
template <class L, class S, bool ODD>
__device__ __forceinline__ void store_edge_populations(const StepParams<S>& P, int x, int y, int z, int i,
                                                       const typename Store<S>::C (&f)[L::Q])
{
#pragma unroll
    for (int p = 0; p < L::Q; ++p) {
        if (ODD) {
            int mx, my, mz;
            nbr_xyz(P.g, x, y, z, L::c(p, 0), L::c(p, 1), L::c(p, 2), mx, my, mz);
            Store<S>::st(P.pop + static_cast<size_t>(p) * P.g.PS + cidx(P.g, mx, my, mz), f[p]);
        } else {
            Store<S>::st(P.pop + static_cast<size_t>(inv<L>(p)) * P.g.PS + i, f[p]);
        }
    }
}

// The step kernel, one launch per time step, with two kinds of blocks.
//
// Row blocks update the bulk and wall cells (kFluidBulk, kFluidWall) of segs<S>() consecutive
// segments of kRowCells cells of x-rows, one thread per cell:
// - At the start the first warp brings the Q source rows of every segment into the segment's own
//   shared-memory stage with bulk asynchronous copies (TMA), one copy per lane, each stage
//   completing on its own mbarrier. Each copied row is the segment widened by 16 bytes on both
//   sides, which keeps source and size 16-byte aligned and covers the +-1 shift in x of the
//   odd-step pulls. The loads in flight are bounded by shared memory rather than registers.
// - While the rows land, each thread loads its flag and link entry (warps of bulk cells only, marked
//   by the segment's warp mask, load neither); FP32 copies the LinkRecords of warps with few linked
//   cells into shared memory.
// - Each cell then collides from the stage and stores its Q populations (store_cell), and the
//   handler values of its links are stored (link_values per lane, or link_values_warp shared by
//   a warp with few linked cells). Handler values sit where the next step pulls them, so no cell
//   needs a special load.
//
// Edge blocks take the cells a row block cannot: a periodic wrap, a free-slip or ghost-fluid
// neighbour, or more handler constants than a record holds. They work from the sorted list
// P.edge, one cell per thread, through global memory (wrapped pulls, store_edge_populations,
// store_handler_values), and are spread over the first part of the grid (see step_kernel).
#ifndef LBMG_ROW_CELLS
#define LBMG_ROW_CELLS 128
#endif
constexpr int kRowCells = LBMG_ROW_CELLS;
// Segments per row block: a block with two segments issues the copies of both at its start, so the
// second segment's rows land while the first one is computed. That pays for 16-bit storage (the
// 256x128x128 D3Q19 channel in FP16: 49.8k against 46.6k MLUPS) and not for FP32 (35.9k against
// 36.4k). LBMG_SEGS sets every storage type in tuning builds.
template <class S>
constexpr int segs()
{
#ifdef LBMG_SEGS
    return LBMG_SEGS;
#else
    return sizeof(S) == 2 ? 2 : 1;
#endif
}
constexpr int kMonFoldThreads = kRowCells;  // threads of a step-kernel block
constexpr uint32_t kMaxPolls = 1u << 20;
// Polls of a row block's first wait for its staged rows. The failure tests build a copy of the
// library with 0 here, so that every such wait gives up at once and runs the give-up path (error
// word, the drain wait with the full limit kMaxPolls, no update of the segment) without any wait
// being left unbounded.
#ifndef LBMG_ROW_WAIT_POLLS
#define LBMG_ROW_WAIT_POLLS (1u << 20)
#endif
constexpr uint32_t kRowWaitPolls = LBMG_ROW_WAIT_POLLS;


template <class S>
constexpr int row_pad()
{
    return static_cast<int>(16 / sizeof(S));
}
// one row-block stage: the widened rows of a segment
template <class L, class S>
constexpr size_t stage_bytes()
{
    const size_t rows = static_cast<size_t>(L::Q) * (kRowCells + 2 * row_pad<S>()) * sizeof(S);
    return (rows + 127) / 128 * 128;
}
// an edge block's handler scratch: the post-collision populations of its cells
template <class L, class S>
constexpr size_t edge_scratch_bytes()
{
    return static_cast<size_t>(L::Q) * kRowCells * sizeof(typename Store<S>::C);
}
// Warps with at most this many kFluidWall cells take the shared handler path (link_values_warp);
// the others (a row along a wall, every lane with links) the per-lane one.
#ifndef LBMG_WARP_LINK_CELLS
#define LBMG_WARP_LINK_CELLS 4
#endif
constexpr int kWarpLinkCells = LBMG_WARP_LINK_CELLS;

// The warp scratch of the shared handler path (link_values_warp): per warp, the Q post-collision
// populations and the 4 moments of each of up to kWarpLinkCells cells.
template <class L, class S>
constexpr size_t warp_scratch_bytes()
{
    return static_cast<size_t>(kRowCells / 32) * kWarpLinkCells * (L::Q + 4) * sizeof(typename Store<S>::C);
}
// The LinkRecords of the shared handler path's cells, copied into shared memory while the rows are
// in flight: kWarpLinkCells per warp (shifted storage). Cells of warps with more linked cells (a
// row along a wall) read theirs from global memory. One record per thread instead took the D3Q19
// FP32 kernel's ten resident blocks past the 196 KB shared-memory carveout, and the smaller L1
// left slowed the edge blocks' gathers by 7% on a periodic box.
// Only FP32 stages them: the 16-bit kernels are issue-bound and ran 1.6% faster on the channel
// reading their few records from global memory, while FP32, latency-bound, gained 1%.
template <class S>
constexpr bool stage_records()
{
    return Store<S>::kShifted && sizeof(S) == 4;
}
template <class S>
constexpr size_t warp_records_bytes()
{
    return stage_records<S>() ? static_cast<size_t>(kRowCells / 32) * kWarpLinkCells * sizeof(LinkRecord) : 0;
}
// Dynamic shared memory of a step-kernel block: a row block's stages, the warp scratch and the
// warp records, or an edge block's scratch from the start, whichever is larger.
template <class L, class S>
constexpr size_t row_smem_bytes()
{
    const size_t rows = segs<S>() * stage_bytes<L, S>() + warp_scratch_bytes<L, S>() + warp_records_bytes<S>();
    const size_t edge = edge_scratch_bytes<L, S>();
    return rows > edge ? rows : edge;
}

// Step monitor. Each block adds the moments its cells started from (m as collide_any returns them,
// accumulated over the block's segments in macc; ncell cells counted) to one of kMonBuckets FP64
// accumulators, one atomic per quantity and block. Shifted storage: m holds rho - 1 and j in FP32,
// values of order 1e-2, so each warp sums them in FP32 (absolute error of order 1e-8 per warp) and
// its lane 0 converts once; the 1 of every counted cell enters as the exact cell count. An FP64
// sum across the lanes costs about 25 FP64 operations per cell, as much time as the whole step at
// this GPU's FP64 rate. FP64 storage keeps FP64 sums. The four warps' sums are added in FP64, in
// a fixed order. Every thread of the block must call it.
template <class S>
__device__ __forceinline__ void monitor_block_add(double* mon, const typename Store<S>::C (&macc)[4], int ncell)
{
    using T = typename Store<S>::C;
    constexpr unsigned full = 0xffffffffu;
    __shared__ double s_part[kMonFoldThreads / 32][4];
    T v[4] = {macc[0], macc[1], macc[2], macc[3]};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] += __shfl_down_sync(full, v[k], o);
    const int n = Store<S>::kShifted ? __reduce_add_sync(full, ncell) : 0;
    if ((threadIdx.x & 31) == 0) {
        s_part[threadIdx.x >> 5][0] = static_cast<double>(v[0]) + static_cast<double>(n);
#pragma unroll
        for (int k = 1; k < 4; ++k) s_part[threadIdx.x >> 5][k] = static_cast<double>(v[k]);
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kMonFoldThreads / 32; ++w) t += s_part[w][threadIdx.x];
        atomicAdd(mon + 4 * (blockIdx.x % kMonBuckets) + threadIdx.x, t);
    }
}

// Sums kMonBuckets x 4 accumulators in a fixed order into out[0..3] and clears them; one block of
// kMonFoldThreads threads. It runs in the first block of the next monitored step (after
// grid_dep_wait, so every addition of the step it folds has completed) or, after the last step,
// in monitor_fold_kernel.
__device__ __forceinline__ void monitor_fold(double* mon, double* out)
{
    __shared__ double s_fold[kMonFoldThreads / 32][4];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = static_cast<int>(threadIdx.x); b < kMonBuckets; b += kMonFoldThreads)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] += __ldcg(mon + 4 * b + k);
            mon[4 * b + k] = 0.0;
        }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if ((threadIdx.x & 31) == 0) s_fold[threadIdx.x >> 5][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
#pragma unroll
        for (int w = 0; w < kMonFoldThreads / 32; ++w) t += s_fold[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

template <class L, class S, bool ODD, bool INSTR>
__device__ __forceinline__ void edge_block(const StepParams<S>& P, int blk, unsigned char* smem_raw,
                                           typename Store<S>::C (&macc)[4], int& ncell)
{
    using St = Store<S>;
    using T = typename St::C;
    constexpr int Q = L::Q;
    const int tx = static_cast<int>(threadIdx.x);
    const int j = blk * kRowCells + tx;
    T m[4] = {T(0), T(0), T(0), T(0)};
    if (j < P.n_edge) {
        const int i = P.edge[j];
        const int r = i - kXOff;
        const int x = r % P.g.XS;
        const int t = r / P.g.XS;
        const int y = t % P.g.YS, z = t / P.g.YS;
        const uint32_t link = P.link[i].x;
        S* __restrict__ pop = P.pop;
        T f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (!ODD) {
                f[q] = St::ld(pop + static_cast<size_t>(q) * P.g.PS + i);
            } else {
                int nx, ny, nz;
                nbr_xyz(P.g, x, y, z, -L::c(q, 0), -L::c(q, 1), -L::c(q, 2), nx, ny, nz);
                f[q] = St::ld(pop + static_cast<size_t>(inv<L>(q)) * P.g.PS + cidx(P.g, nx, ny, nz));
            }
        }
        collide_any<L, S>(f, P, m);
        if (INSTR && P.rec) record_moments<S>(P.rec, i, m);
        store_edge_populations<L, S, ODD>(P, x, y, z, i, f);
        if (link & ((1u << Q) - 1u)) {
            T* fs = reinterpret_cast<T*>(smem_raw) + tx;
#pragma unroll
            for (int q = 0; q < Q; ++q) fs[q * kRowCells] = f[q];
            store_handler_values<L, S, ODD>(P, x, y, z, i, link, fs, kRowCells);
        }
    }
    if constexpr (INSTR) {
#pragma unroll
        for (int k = 0; k < 4; ++k) macc[k] += m[k];
        ncell += j < P.n_edge;
    }
}

__device__ __forceinline__ void segment_origin(const Geom& g, int seg, const FastDiv& dx, const FastDiv& dy, int& x0,
                                               int& y, int& z)
{
    const uint32_t yz = fast_div(static_cast<uint32_t>(seg), dx);
    x0 = 1 + (seg - static_cast<int>(yz * dx.d)) * kRowCells;
    const uint32_t zz = fast_div(yz, dy);
    y = 1 + static_cast<int>(yz - zz * dy.d);
    z = 1 + static_cast<int>(zz);
}

// Handler values of a kFluidWall cell, after its collision. For every link ip = inv(p) (x + c_p
// is a handler cell m) the cell stores m's handler value B_ip where it pulls it next step: after
// an odd step slot ip at x, after an even step plane p at m. B_ip: no-slip f*_p; moving wall
// f*_p + c rho; inflow c; outflow / pressure feq_ip(r0, j/r0) + feq_p(r0, j/r0) - f*_p, in
// shifted form 2 w_p (r0 - 1 + r0 (cu_p^2 / (2 cs4) - |u|^2 / (2 cs2))) - f*_p (the odd terms
// cancel), from the cell's LinkRecord rec (shifted storage only). ps and gy are the plane stride
// and XS, hidden from the optimiser so that this path's address arithmetic stays in it.
template <class L, class S, bool ODD>
__device__ __forceinline__ void link_values(const StepParams<S>& P, int i, typename Store<S>::C (&f)[L::Q],
                                            const typename Store<S>::C (&m)[4], uint32_t wl,
                                            const uint32_t* rec, size_t ps, int gy)
{
    using St = Store<S>;
    using T = typename St::C;
    constexpr int Q = L::Q;
    S* own = P.pop + i;
    uint32_t spec = 0, valm = 0, wallm = 0;
    float r0 = 1.f, ux = 0.f, uy = 0.f, uz = 0.f, uu_c = 0.f, rho = 1.f;
    if constexpr (St::kShifted) {
        if (rec) {
            spec = rec[0];
            wallm = rec[1];
            valm = wallm | rec[2];
            r0 = __uint_as_float(rec[3]);
            const float ir0 = __uint_as_float(rec[4]);
            ux = m[1] * ir0;
            uy = m[2] * ir0;
            uz = m[3] * ir0;
            uu_c = (ux * ux + uy * uy + uz * uz) * kC;
            rho = 1.f + m[0];
        }
    }
#pragma unroll
    for (int p = 0; p < Q; ++p) {
        const int ip = inv<L>(p);
        if (!((wl >> ip) & 1u)) continue;
        T v = f[p];
        if constexpr (St::kShifted) {
            if ((spec >> ip) & 1u) {
                if ((valm >> ip) & 1u) {
                    const int k = min(__popc(valm & ((1u << ip) - 1u)), kMaxRecordValues - 1);
                    const float c = __uint_as_float(rec[5 + k]);
                    v = ((wallm >> ip) & 1u) ? fmaf(c, rho, f[p]) : c;
                } else {
                    const float cu = L::c(p, 0) * ux + L::c(p, 1) * uy + L::c(p, 2) * uz;
                    v = 2.f * static_cast<float>(L::w(p)) * ((r0 - 1.f) + r0 * fmaf(cu * cu, kB, -uu_c)) - f[p];
                }
            }
        }
        if (ODD) {
            St::st(own + static_cast<size_t>(ip) * ps, v);
        } else {
            const int off = L::c(p, 0) + L::c(p, 1) * gy + L::c(p, 2) * gy * P.g.YS;
            St::st(own + static_cast<size_t>(p) * ps + off, v);
        }
    }
}

// Handler values (as link_values) of the kFluidWall cells of a warp that holds only a few of them,
// typically the one cell next to an inlet or outlet at the end of a row, whose per-lane path would
// hold the other 31 lanes for its whole length. Each such cell (a source lane, the k-th lane of
// `need`) has put its post-collision populations and moments into slot k of the warp's scratch
// (warp_link_source), and its LinkRecord, if it has one (row), is slot k of recs where records are
// staged (stage_records), else row `row` of ltab; here, per source, lane ip stores the value of
// link ip. Every lane of the warp calls it with the same `need` (at most kWarpLinkCells lanes with
// links); wl is 0 on the other lanes. Same operations per value as link_values.
template <class L, class S, bool ODD>
__device__ __forceinline__ void link_values_warp(S* pop, unsigned need, int i, uint32_t wl, uint32_t row,
                                              const LinkRecord* recs, const LinkRecord* ltab,
                                              const typename Store<S>::C* scr, size_t ps, int sy, int sz)
{
    using St = Store<S>;
    using T = typename St::C;
    constexpr int Q = L::Q;
    constexpr int SW = Q + 4;  // scratch words of one source
    constexpr unsigned kFull = 0xffffffffu;
    const int ip = static_cast<int>(threadIdx.x & 31u);  // this lane's link
    for (unsigned rem = need; rem; rem &= rem - 1u, scr += SW, ++recs) {
        const int src = __ffs(rem) - 1;
        const uint32_t swl = __shfl_sync(kFull, wl, src);
        const int si = __shfl_sync(kFull, i, src);
        const uint32_t srow = __shfl_sync(kFull, row, src);  // the source's LinkRecord row
        if (ip < Q && ((swl >> ip) & 1u)) {
            // direction p = inv(ip): after an odd step slot ip at the source cell x, after an even
            // step plane p at x + c_p
            const int p = Q - 1 - ip;
            const int cx = rt_c<L>(p, 0), cy = rt_c<L>(p, 1), cz = rt_c<L>(p, 2);
            T v = scr[p];
            if constexpr (St::kShifted) {
                const uint32_t* r = reinterpret_cast<const uint32_t*>(stage_records<S>() ? recs : ltab + srow);
                if (srow != kNoRecord && ((r[0] >> ip) & 1u)) {
                    const uint32_t wallm = r[1], valm = wallm | r[2];
                    if ((valm >> ip) & 1u) {
                        const int k = min(__popc(valm & ((1u << ip) - 1u)), kMaxRecordValues - 1);
                        const float c = __uint_as_float(r[5 + k]);
                        v = ((wallm >> ip) & 1u) ? fmaf(c, 1.f + scr[Q], v) : c;
                    } else {
                        const float r0 = __uint_as_float(r[3]), ir0 = __uint_as_float(r[4]);
                        const float ux = scr[Q + 1] * ir0, uy = scr[Q + 2] * ir0, uz = scr[Q + 3] * ir0;
                        const float uu_c = (ux * ux + uy * uy + uz * uz) * kC;
                        const float cu = static_cast<float>(cx) * ux + static_cast<float>(cy) * uy +
                                         static_cast<float>(cz) * uz;
                        v = 2.f * static_cast<float>(rt_w<L>(p)) * ((r0 - 1.f) + r0 * fmaf(cu * cu, kB, -uu_c)) - v;
                    }
                }
            }
            const long long off = ODD ? static_cast<long long>(ip) * static_cast<long long>(ps)
                                      : static_cast<long long>(p) * static_cast<long long>(ps) +
                                            (cx + cy * sy + cz * sz);
            St::st(pop + si + off, v);
        }
    }
}

// A source lane of link_values_warp: its populations and moments into its slot of the scratch.
template <class L, class S>
__device__ __forceinline__ void warp_link_source(unsigned need, const typename Store<S>::C (&f)[L::Q],
                                                 const typename Store<S>::C (&m)[4], typename Store<S>::C* scr)
{
    constexpr int Q = L::Q;
    const unsigned lane = threadIdx.x & 31u;
    typename Store<S>::C* mine = scr + (Q + 4) * __popc(need & ((1u << lane) - 1u));
#pragma unroll
    for (int q = 0; q < Q; ++q) mine[q] = f[q];
#pragma unroll
    for (int k = 0; k < 4; ++k) mine[Q + k] = m[k];
}

// The Q bulk stores of a row-block cell at layout pointer `cell`, plane by plane through one
// running pointer (each step adds a block-uniform delta: the plane stride and, on odd steps, the
// change of the shift c_p).
template <class L, class S, bool ODD, bool STREAM>
__device__ __forceinline__ void store_cell(S* cell, const typename Store<S>::C (&f)[L::Q], size_t PS, int sy, int sz)
{
    using St = Store<S>;
    constexpr int Q = L::Q;
    if (ODD) {
        S* ptr = cell + (L::c(0, 0) + L::c(0, 1) * sy + L::c(0, 2) * sz);
#pragma unroll
        for (int p = 0; p < Q; ++p) {
            if (STREAM) St::st_stream(ptr, f[p]); else St::st(ptr, f[p]);
            if (p + 1 < Q) {
                const int d = (L::c(p + 1, 0) - L::c(p, 0)) + (L::c(p + 1, 1) - L::c(p, 1)) * sy +
                              (L::c(p + 1, 2) - L::c(p, 2)) * sz;
                ptr += static_cast<long long>(PS) + d;
            }
        }
    } else {
        S* ptr = cell;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            if (STREAM) St::st_stream(ptr, f[inv<L>(k)]); else St::st(ptr, f[inv<L>(k)]);
            if (k + 1 < Q) ptr += PS;
        }
    }
}

// The value v, hidden from the optimiser: address arithmetic that uses it stays inside the
// (rarely taken) branch it is written in instead of being hoisted into registers held by every
// thread of the kernel.
template <class V>
__device__ __forceinline__ V opaque(V v)
{
    if constexpr (sizeof(V) == 8)
        asm volatile("" : "+l"(v));
    else
        asm volatile("" : "+r"(v));
    return v;
}

// LINKS: the handler path is compiled in (domains with handler cells). Without it a kFluidWall cell
// would lose its handler values, so a domain without handler cells, which has none, is the only
// user of LINKS = false (see the step launcher).
template <class L, class S, bool ODD, bool INSTR, bool LINKS>
__device__ __forceinline__ void row_block(const StepParams<S>& P, int rb, int nseg, const FastDiv& dx, const FastDiv& dy,
                                          unsigned char* smem_raw, uint64_t* bars, typename Store<S>::C (&macc)[4],
                                          int& ncell)
{
    using St = Store<S>;
    using T = typename St::C;
    constexpr int Q = L::Q;
    constexpr int PAD = row_pad<S>();
    constexpr int W = kRowCells + 2 * PAD;
    constexpr size_t SB = stage_bytes<L, S>();
    constexpr uint32_t bytes = W * sizeof(S);
    const int tx = static_cast<int>(threadIdx.x);
    const size_t PS = P.g.PS;
    S* __restrict__ pop = P.pop;
    constexpr int kSegs = segs<S>();
    const int seg0 = rb * kSegs;
    const int nsegs = nseg - seg0 < kSegs ? nseg - seg0 : kSegs;

    if (tx == 0) {
#pragma unroll
        for (int s = 0; s < kSegs; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tx < 32) {
        const int lane = tx;
        for (int s = 0; s < nsegs; ++s) {
            int x0, y, z;
            segment_origin(P.g, seg0 + s, dx, dy, x0, y, z);
            if (lane == 0) mbar_arrive_expect_tx(&bars[s], Q * bytes);
            __syncwarp();
            if (lane < Q) {
                // bulk cells never pull across a periodic wrap, so no source row needs wrapping
                const int q = lane;
                const int plane = ODD ? inv<L>(q) : q;
                const int ry = ODD ? y - rt_c<L>(q, 1) : y;
                const int rz = ODD ? z - rt_c<L>(q, 2) : z;
                const S* src = pop + static_cast<size_t>(plane) * PS +
                               (static_cast<size_t>(kXOff + x0 - PAD) +
                                static_cast<size_t>(P.g.XS) * (static_cast<size_t>(ry) + static_cast<size_t>(P.g.YS) * rz));
                bulk_g2s_hint(reinterpret_cast<S*>(smem_raw + s * SB) + q * W, src, bytes, &bars[s],
                              l2_stream_policy(P.n_edge == 0));
            }
        }
    }
    const int sy = P.g.XS;
    const int sz = P.g.XS * P.g.YS;
    for (int s = 0; s < nsegs; ++s) {
        int x0, y, z;
        segment_origin(P.g, seg0 + s, dx, dy, x0, y, z);
        const int x = x0 + tx;
        const int i = cidx(P.g, x, y, z);
        // links of a kFluidWall cell (bit q: x - c_q is a no-slip, moving-wall, inflow, outflow
        // or pressure cell), and its LinkRecord, copied into shared memory while the rows are in
        // flight (shifted storage). Cells on a face of the domain, where boundaries usually sit,
        // load their link word together with their flag instead of after it. A warp whose cells
        // are all kFluidBulk (the segment's warp mask) loads neither.
        bool bulk = true;
        uint2 lk = make_uint2(0u, kNoRecord);
        LinkRecord* recs = reinterpret_cast<LinkRecord*>(smem_raw + kSegs * SB + warp_scratch_bytes<L, S>()) +
                           (tx >> 5) * kWarpLinkCells;
        bool staged = false;
        if (!((P.wmask[seg0 + s] >> (tx >> 5)) & 1u)) {  // (warp-uniform)
            const bool face = x == 1 || x == P.g.xl || y == 1 || y == P.g.yl || z == 1 || z == P.g.zl;
            const uint2 lkf = face && x <= P.g.xl ? P.link[i] : make_uint2(0u, kNoRecord);
            const uint8_t fl = x <= P.g.xl ? P.flag[i] : static_cast<uint8_t>(kFluidEdge);
            bulk = fl == kFluidBulk || fl == kFluidWall;
            lk = fl != kFluidWall ? make_uint2(0u, kNoRecord) : face ? lkf : P.link[i];
            // the cell's LinkRecord (shifted storage): in a warp with few linked cells copied into
            // the warp's record slot (the cell's rank among them) while the rows are in flight, else
            // read from global memory where it is used (fetched into L1 now)
            if constexpr (St::kShifted && LINKS) {
                const unsigned need_e = stage_records<S>() ? __ballot_sync(0xffffffffu, lk.x != 0u) : ~0u;
                if (lk.y != kNoRecord) {
                    const char* src = reinterpret_cast<const char*>(P.ltab + lk.y);
                    if (stage_records<S>() && __popc(need_e) <= kWarpLinkCells) {
                        char* dst = reinterpret_cast<char*>(recs + __popc(need_e & ((1u << (tx & 31)) - 1u)));
#pragma unroll
                        for (int w = 0; w < static_cast<int>(sizeof(LinkRecord) / 16); ++w)
                            cp_async16(dst + 16 * w, src + 16 * w);
                        cp_async_commit();
                        staged = true;
                    } else {
                        prefetch_l1(src);
                    }
                }
            }
        }
        const uint32_t wl = lk.x;
        const uint32_t* rec = St::kShifted && lk.y != kNoRecord
                                  ? reinterpret_cast<const uint32_t*>(P.ltab + lk.y) : nullptr;
        if (!mbar_wait_bounded(&bars[s], 0, kRowWaitPolls)) {
            // the step's results are invalid; still never leave while copies may land here (this
            // drain wait is bounded too: if it also gives up the block returns regardless)
            *P.err = 1;
            mbar_wait_bounded(&bars[s], 0, kMaxPolls);
            bulk = false;
        }
        T m[4] = {T(0), T(0), T(0), T(0)};
        T f[Q];
        if (bulk) {
            const S* buf = reinterpret_cast<const S*>(smem_raw + s * SB);
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q] = St::ld(buf + q * W + PAD + tx - (ODD ? L::c(q, 0) : 0));
            collide_any<L, S>(f, P, m);
            if (INSTR && P.rec) record_moments<S>(P.rec, i, m);
            // stores plane by plane through one running pointer: each step adds a block-uniform
            // delta (the plane stride, and on odd steps the change of the shift c_p). Streaming
            // (evict-first) stores when every cell is a row-block cell (see l2_stream_policy).
            if (P.n_edge == 0)
                store_cell<L, S, ODD, true>(pop + i, f, PS, sy, sz);
            else
                store_cell<L, S, ODD, false>(pop + i, f, PS, sy, sz);
        }
        // handler values, into slots that no cell's own stores touch: shared by the warp when
        // few of its cells have links, else per lane
        const uint32_t wlb = LINKS && bulk ? wl : 0u;
        const unsigned need = LINKS ? __ballot_sync(0xffffffffu, wlb != 0u) : 0u;
        if (LINKS && need) {
            // (need equals need_e unless the row wait gave up, which leaves need empty)
            if (__popc(need) <= kWarpLinkCells) {
                T* scr = reinterpret_cast<T*>(smem_raw + kSegs * SB) + (tx >> 5) * kWarpLinkCells * (Q + 4);
                if (wlb) {
                    if (staged) cp_async_wait_all();  // this lane's record has landed
                    warp_link_source<L, S>(need, f, m, scr);
                }
                __syncwarp();
                link_values_warp<L, S, ODD>(pop, need, i, wlb, lk.y, recs, P.ltab, scr, PS, sy, sz);
                __syncwarp();  // scratch and records are read before the warp's next segment writes them
            } else if (wlb) {
                link_values<L, S, ODD>(P, i, f, m, wlb, rec, opaque(PS), opaque(sy));
            }
        }
        if (staged) cp_async_wait_all();  // no copy may still be landing when the block ends
        if constexpr (INSTR) {
#pragma unroll
            for (int k = 0; k < 4; ++k) macc[k] += m[k];
            ncell += bulk;
        }
    }
}

// Resident blocks per SM that the register allocation of a step kernel must allow (0: no
// bound; ptxas then picks fewer registers than with an explicit 1). Shifted D3Q19 kernels: 10
// blocks (48 registers; unbounded they take 56, 9 blocks). D3Q15: 12 blocks (40 registers) for
// FP32 (46.5k against 45.4k MLUPS at 10 on the 256x128x128 channel), 10 for 16-bit storage (67.3k
// against 65.3k at 12, where the 40-register kernels spill). D3Q27: 7 blocks for FP32 (72
// registers; 24.2k against 23.9k unbounded at 72-80 and 23.9k at 8) and 8 blocks for 16-bit
// storage (64 registers; 40.3k against 38.7k unbounded). FP64 is never bounded. LBMG_MINB_Q15 / LBMG_MINB_Q27 set the D3Q15
// and D3Q27 values of every storage type, LBMG_MINB_EVEN / LBMG_MINB_ODD the shifted-storage
// values, in tuning builds.
template <class L, class S, bool ODD, bool INSTR>
constexpr int min_blocks()
{
    if constexpr (!Store<S>::kShifted) {
        return 0;
    } else {
#if defined(LBMG_MINB_ODD)
        if (ODD) return LBMG_MINB_ODD;
#endif
#if defined(LBMG_MINB_EVEN)
        if (!ODD) return LBMG_MINB_EVEN;
#endif
        // the instrumented kernels (monitor, adjoint record) would spill at the plain kernels'
        // bounds: D3Q15 at 40 registers, D3Q19 at 48
        if (INSTR && L::Q == 15) return 10;
        if (INSTR && L::Q == 19) return 9;
        constexpr bool k16 = sizeof(S) == 2;
        if (L::Q == 19) return 10;
#ifdef LBMG_MINB_Q15
        if (L::Q == 15) return LBMG_MINB_Q15;
#endif
#ifdef LBMG_MINB_Q27
        if (L::Q == 27) return LBMG_MINB_Q27;
#endif
        if (L::Q == 15) return k16 ? 10 : 12;
        return k16 ? 8 : 7;
    }
}

// Edge blocks sit at every `edge_stride`-th block index (the first n_edge_blocks such
// positions), so that the latency-bound edge work is spread over the first part of the launch
// instead of holding the SMs at its start or running on after the last row block; the row
// blocks fill the other indices in order.
#ifndef LBMG_EDGE_SPAN
#define LBMG_EDGE_SPAN 0.6
#endif
constexpr double kEdgeSpan = LBMG_EDGE_SPAN;
// INSTR: the step monitor and the adjoint's record may be active (P.mon / P.rec are tested);
// plain steps are compiled without them.
template <class L, class S, bool ODD, bool INSTR, bool LINKS>
__global__ void __launch_bounds__(kRowCells, min_blocks<L, S, ODD, INSTR>())
    step_kernel(const StepParams<S> P, int n_edge_blocks, FastDiv edge_stride, int nseg, FastDiv nseg_x, FastDiv yl)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[segs<S>()];
    // before any global access: the previous step (or whatever kernel precedes this one) has
    // completed; then the next step's blocks may take the SMs this grid's last blocks leave
    grid_dep_wait();
    grid_dep_launch();
    const int b = static_cast<int>(blockIdx.x);
    if constexpr (INSTR) {
        if (P.mon_prev && b == 0) monitor_fold(P.mon_prev, P.mon_prev_out);
    }
    using T = typename Store<S>::C;
    T macc[4] = {T(0), T(0), T(0), T(0)};
    int ncell = 0;
    const int interleaved = n_edge_blocks * static_cast<int>(edge_stride.d);
    const int e = static_cast<int>(fast_div(static_cast<uint32_t>(b), edge_stride));
    if (b < interleaved && b == e * static_cast<int>(edge_stride.d))
        edge_block<L, S, ODD, INSTR>(P, e, smem_raw, macc, ncell);
    else if (b < interleaved)
        row_block<L, S, ODD, INSTR, LINKS>(P, b - (e + 1), nseg, nseg_x, yl, smem_raw, bars, macc, ncell);
    else
        row_block<L, S, ODD, INSTR, LINKS>(P, b - n_edge_blocks, nseg, nseg_x, yl, smem_raw, bars, macc, ncell);
    if constexpr (INSTR) {
        if (P.mon) monitor_block_add<S>(P.mon, macc, ncell);
    }
}

// The fold of the last monitored step of a call (see monitor_fold).
static __global__ void __launch_bounds__(kMonFoldThreads) monitor_fold_kernel(double* mon, double* out)
{
    monitor_fold(mon, out);
}

// ------------------------------------------------------------------------------------------
// Reading the state back in the reference's terms.
// ------------------------------------------------------------------------------------------

// Post-collision population p of interior fluid cell (x, y, z) at layout index i, after a
// number of steps whose parity is `odd`.
template <class L, class S>
__device__ __forceinline__ typename Store<S>::C load_post(const S* pop, const uint8_t* flag,
                                                          const Geom& g, int x, int y, int z,
                                                          int i, int p, bool odd)
{
    if (!odd) return Store<S>::ld(pop + static_cast<size_t>(inv<L>(p)) * g.PS + i);
    int mx, my, mz;
    nbr_xyz(g, x, y, z, L::c(p, 0), L::c(p, 1), L::c(p, 2), mx, my, mz);
    return Store<S>::ld(pop + static_cast<size_t>(p) * g.PS + cidx(g, mx, my, mz));
}

// collide_field populations of any cell as FP64 (see lbm_get_populations). Ghost-fluid cells
// come out as w_q here; the caller overwrites them from the side copies.
template <class L, class S>
__device__ __forceinline__ void load_cell_f64(const S* pop, const uint8_t* flag, const Geom& g,
                                              int x, int y, int z, bool odd, double (&out)[L::Q])
{
    const int i = cidx(g, x, y, z);
    const uint8_t fl = flag[i];
    if (is_fluid(fl) && interior(g, x, y, z)) {
#pragma unroll
        for (int p = 0; p < L::Q; ++p)
            out[p] = to_f64<L, S>(load_post<L, S>(pop, flag, g, x, y, z, i, p, odd), p);
        return;
    }
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, L::c(q, 0), L::c(q, 1), L::c(q, 2), nx, ny, nz);
        double v = L::w(q);
        if (fl >= kFirstHandler && interior(g, nx, ny, nz)) {
            const int n = cidx(g, nx, ny, nz);
            if (is_fluid(flag[n]))
                v = to_f64<L, S>(odd ? Store<S>::ld(pop + static_cast<size_t>(q) * g.PS + n)
                                     : Store<S>::ld(pop + static_cast<size_t>(inv<L>(q)) * g.PS + i),
                                 q);
        }
        out[q] = v;
    }
}

}  // namespace lbmg
