// Lattice models D3Q15 / D3Q19 / D3Q27 as compile-time tables.
//
// Velocity orderings and weights are the reference's (model.h:13-50, 53-91, 96-139): the
// population index q means the same direction here and there, which population-level parity
// and the Q-1-q opposite rule (model.h:36-39) depend on. Every table lookup below is folded
// by the compiler once the q-loops are unrolled, so the kernels carry no table in memory.
#pragma once

#include <cstdint>

#include "divrn.cuh"

namespace lbmg {

// lbmdefinitions.h:47 defines C_S as 0.57735026919l converted to double; this hex literal is
// that double (0x3fe279a745904047). Its square differs from 1/3 by 4.3e-13, which the FP64 path
// keeps so that it reproduces the reference to the last bit.
constexpr double kCS = 0x1.279a745904047p-1;
constexpr double kCS2 = kCS * kCS;                     // C_S * C_S          (collision.hpp:45)
constexpr double kCS4x2 = 2 * kCS * kCS * kCS * kCS;   // 2*C_S*C_S*C_S*C_S  (collision.hpp:45)
constexpr double kCS2x2 = 2 * kCS * kCS;               // 2*C_S*C_S          (collision.hpp:46)
// The three divisors with their reciprocal pairs {y, RN(1/y), RN((1 - y RN(1/y)) / y)} for
// div_rn (divrn.cuh); the host check tests/cpp/div_rn_check.cpp recomputes them.
__host__ __device__ constexpr DivRN cs2_div() { return {kCS2, 0x1.7ffffffffddcap+1, 0x1.000000c30db6dp-53}; }
__host__ __device__ constexpr DivRN cs4x2_div() { return {kCS4x2, 0x1.1ffffffffccb0p+2, -0x1.17fffdb6dee01p-52}; }
__host__ __device__ constexpr DivRN cs2x2_div() { return {kCS2x2, 0x1.7ffffffffddcap+0, 0x1.000000c30db6dp-54}; }

template <int QQ>
struct Lattice;

template <>
struct Lattice<15> {
    static constexpr int Q = 15;
    static constexpr int REST = 7;
    __host__ __device__ static constexpr int c(int q, int d)
    {
        constexpr signed char t[15][3] = {
            {-1, -1, -1}, {1, -1, -1}, {0, 0, -1}, {-1, 1, -1}, {1, 1, -1},
            {0, -1, 0},   {-1, 0, 0},  {0, 0, 0},  {1, 0, 0},   {0, 1, 0},
            {-1, -1, 1},  {1, -1, 1},  {0, 0, 1},  {-1, 1, 1},  {1, 1, 1}};
        return t[q][d];
    }
    __host__ __device__ static constexpr double w(int q)
    {
        constexpr double t[15] = {1.0 / 72, 1.0 / 72,  8.0 / 72, 1.0 / 72, 1.0 / 72,
                                  8.0 / 72, 8.0 / 72, 16.0 / 72, 8.0 / 72, 8.0 / 72,
                                  1.0 / 72, 1.0 / 72,  8.0 / 72, 1.0 / 72, 1.0 / 72};
        return t[q];
    }
    // model.h:41-44
    __host__ __device__ static constexpr int velocity_index(int u, int v, int w)
    {
        return 5 * w + 2 * v + u + 7 - (w + 2) % 2 * (u + v) / 2;
    }
};

template <>
struct Lattice<19> {
    static constexpr int Q = 19;
    static constexpr int REST = 9;
    __host__ __device__ static constexpr int c(int q, int d)
    {
        constexpr signed char t[19][3] = {
            {0, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {0, 1, -1},
            {-1, -1, 0}, {0, -1, 0},  {1, -1, 0}, {-1, 0, 0}, {0, 0, 0},
            {1, 0, 0},   {-1, 1, 0},  {0, 1, 0},  {1, 1, 0},  {0, -1, 1},
            {-1, 0, 1},  {0, 0, 1},   {1, 0, 1},  {0, 1, 1}};
        return t[q][d];
    }
    __host__ __device__ static constexpr double w(int q)
    {
        constexpr double t[19] = {1.0 / 36, 1.0 / 36, 2.0 / 36, 1.0 / 36, 1.0 / 36,
                                  1.0 / 36, 2.0 / 36, 1.0 / 36, 2.0 / 36, 12.0 / 36,
                                  2.0 / 36, 1.0 / 36, 2.0 / 36, 1.0 / 36, 1.0 / 36,
                                  1.0 / 36, 2.0 / 36, 1.0 / 36, 1.0 / 36};
        return t[q];
    }
    // model.h:82-85
    __host__ __device__ static constexpr int velocity_index(int u, int v, int w)
    {
        return w == 0 ? (6 + (v + 1) * 3 + u) : ((w + 1) * 7 + (v + 1) * 2 + u);
    }
};

template <>
struct Lattice<27> {
    static constexpr int Q = 27;
    static constexpr int REST = 13;
    __host__ __device__ static constexpr int c(int q, int d)
    {
        // z outer, y middle, x inner: c = (q%3-1, (q/3)%3-1, q/9-1) (model.h:103-111)
        return d == 0 ? q % 3 - 1 : (d == 1 ? (q / 3) % 3 - 1 : q / 9 - 1);
    }
    __host__ __device__ static constexpr double w(int q)
    {
        constexpr double t[27] = {
            1.0 / 216,  4.0 / 216, 1.0 / 216,  4.0 / 216,  16.0 / 216, 4.0 / 216,  1.0 / 216,
            4.0 / 216,  1.0 / 216, 4.0 / 216,  16.0 / 216, 4.0 / 216,  16.0 / 216, 64.0 / 216,
            16.0 / 216, 4.0 / 216, 16.0 / 216, 4.0 / 216,  1.0 / 216,  4.0 / 216,  1.0 / 216,
            4.0 / 216,  16.0 / 216, 4.0 / 216, 1.0 / 216,  4.0 / 216,  1.0 / 216};
        return t[q];
    }
    // model.h:130-133
    __host__ __device__ static constexpr int velocity_index(int u, int v, int w)
    {
        return 9 * w + 3 * v + u + 13;
    }
};

// Opposite direction: Q-1-q for all three models (model.h:36-39, 77-80, 124-127).
template <class L>
__host__ __device__ constexpr int inv(int q)
{
    return L::Q - 1 - q;
}

// Velocity components and weights for a direction index known only at run time, without a
// table in memory: each component is packed as 2 bits (c + 1) into compile-time constants, and
// each weight as a 2-bit class (one of at most four distinct weights).
template <class L>
struct Packed {
    static constexpr uint64_t bits(int lo, int hi)
    {
        uint64_t v = 0;
        for (int k = lo; k < hi && k < 3 * L::Q; ++k)
            v |= static_cast<uint64_t>(L::c(k / 3, k % 3) + 1) << (2 * (k - lo));
        return v;
    }
    static constexpr uint64_t kC0 = bits(0, 32);   // components 0..31
    static constexpr uint64_t kC1 = bits(32, 64);  // components 32..63
    static constexpr uint64_t kC2 = bits(64, 96);  // components 64..80
    // representative direction of each weight class (at most four distinct weights)
    static constexpr int kRep0 = 0;
    static constexpr int kRep1 = L::Q == 15 ? 2 : (L::Q == 19 ? 2 : 1);
    static constexpr int kRep2 = L::Q == 15 ? 7 : (L::Q == 19 ? 9 : 4);
    static constexpr int kRep3 = L::Q == 27 ? 13 : kRep2;
    static constexpr int wclass(double w)
    {
        return w == L::w(kRep0) ? 0 : (w == L::w(kRep1) ? 1 : (w == L::w(kRep2) ? 2 : 3));
    }
    static constexpr uint64_t wbits()
    {
        uint64_t v = 0;
        for (int q = 0; q < L::Q; ++q) v |= static_cast<uint64_t>(wclass(L::w(q))) << (2 * q);
        return v;
    }
    static constexpr uint64_t kWC = wbits();
};

template <class L>
__host__ __device__ __forceinline__ int rt_c(int q, int d)
{
    const int k = 3 * q + d;
    const uint64_t word = k < 32 ? Packed<L>::kC0 : (k < 64 ? Packed<L>::kC1 : Packed<L>::kC2);
    return static_cast<int>((word >> (2 * (k & 31))) & 3u) - 1;
}

template <class L>
__host__ __device__ __forceinline__ double rt_w(int q)
{
    const int cls = static_cast<int>((Packed<L>::kWC >> (2 * q)) & 3u);
    return cls == 0 ? L::w(Packed<L>::kRep0)
                    : (cls == 1 ? L::w(Packed<L>::kRep1) : (cls == 2 ? L::w(Packed<L>::kRep2) : L::w(Packed<L>::kRep3)));
}

}  // namespace lbmg
