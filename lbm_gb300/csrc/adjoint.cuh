// Discrete adjoint of the time step (an extension: the reference has no gradients).
//
// Forward step t (cell x, direction q): the pulled population g_t,q(x) is the neighbour's
// post-collision f*_{t-1,q}(x - c_q), or, when x - c_q is a boundary cell, that cell's handler
// value B_q(f*_{t-1}(x), theta) (theta: wall or inflow velocity), evaluated at the end of step
// t-1; f*_t(x) = BGK(g_t(x)). The boundary values that the first step of a run pulls belong to the
// state the run starts from (the initial values at step 1: the reference runs no handler before its
// first stream), so over steps s0+1 .. s0+n theta enters through steps s0+2 .. s0+n.
//
// With lambda_t = dJ/df*_t and mu_t = dJ/dg_t the adjoint step is, per fluid cell x,
//   lambda_{t-1}(x)_p = mu_t(x + c_p)_p                    (x + c_p fluid; the transposed pull)
//                     + sum_{q: x - c_q boundary} mu_t(x)_q dB_q/df*_p      (t >= 2)
//   mu_{t-1}(x)       = J_BGK(g_{t-1}(x))^T lambda_{t-1}(x)
// and dJ/dtheta += sum_{t >= s0+2} sum_{x, q} mu_t(x)_q dB_q/dtheta. The BGK Jacobian depends on
// g only through its mass and momentum, which the recompute segments record per cell (the same
// as the post-collision ones: BGK conserves them), so the adjoint reads 4 values per cell and
// step besides the Q adjoint populations.
#pragma once

#include "kernels.cuh"
#include "state_kernels.cuh"  // kReduceThreads

namespace lbmg {

template <class T>
struct AdjParams {
    const uint8_t* flag;
    const uint2* link;
    const LinkRecord* ltab;  // handler records of kFluidWall cells (shifted storage), or nullptr
    const BcEntry* bc;
    const double* profile;
    Geom g;
    T omega;
    const T* mu_in;       // mu_t, Q planes of PS
    T* mu_out;            // mu_{t-1}
    const T* rec;         // mass and momentum of g_{t-1}, 4 per cell (layout index), 16-byte aligned
    int bc_terms;         // 1: the handler terms of step t apply (t >= s0 + 2)
    int write_mu;         // 0: only the theta gradients of step t
    double* grad_inflow;  // 3 per cell, reference cell order (inflow cells)
    double* grad_wall;    // 3 per handler
};

template <class T>
struct AdjConst;
template <>
struct AdjConst<float> {
    static constexpr float A = kA, B = kB, C = kC;
};
template <>
struct AdjConst<double> {
    static constexpr double A = 1.0 / kCS2, B = 1.0 / kCS4x2, C = 1.0 / kCS2x2;
};

// acc += s * v for a lattice component s in {-1, 0, 1} (a constant once the loops are unrolled).
template <class T>
__host__ __device__ __forceinline__ void add_signed(T& acc, T v, int s)
{
    if (s > 0) acc += v;
    else if (s < 0) acc -= v;
}

// In place: lam <- J^T lam for the BGK map at a state of mass rho and momentum j:
//   J = (1 - omega) I + omega d feq / dg,  feq_q = w_q rho (1 + A cu + B cu^2 - C uu).
// (J^T lam)_p = (1 - omega) lam_p + omega (s0 + (c_p - u) . V) with
//   s0 = sum_q w_q lam_q (1 + A cu_q + B cu_q^2 - C uu),
//   V  = sum_q w_q lam_q ((A + 2 B cu_q) c_q - 2 C u),
// and both depend on lam only through its ten weighted moments a = sum w lam, b = sum w lam c and
// M = sum w lam c c^T: s0 = a (1 - C uu) + A u.b + B u.M u, V = A b + 2 B M u - 2 C a u. So the
// per-direction work is signed adds (c has components -1, 0, 1) and one multiply-add.
template <class L, class T>
__host__ __device__ __forceinline__ void bgk_adjoint(T (&lam)[L::Q], T rho, T jx, T jy, T jz, T omega)
{
    using K = AdjConst<T>;
    const T ir = T(1) / rho;
    const T ux = jx * ir, uy = jy * ir, uz = jz * ir;
    const T uu = ux * ux + uy * uy + uz * uz;
    T a = 0, bx = 0, by = 0, bz = 0, mxx = 0, myy = 0, mzz = 0, mxy = 0, mxz = 0, myz = 0;
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        const int cx = L::c(q, 0), cy = L::c(q, 1), cz = L::c(q, 2);
        const T lw = lam[q] * T(L::w(q));
        a += lw;
        add_signed(bx, lw, cx);
        add_signed(by, lw, cy);
        add_signed(bz, lw, cz);
        add_signed(mxx, lw, cx * cx);
        add_signed(myy, lw, cy * cy);
        add_signed(mzz, lw, cz * cz);
        add_signed(mxy, lw, cx * cy);
        add_signed(mxz, lw, cx * cz);
        add_signed(myz, lw, cy * cz);
    }
    const T mux = mxx * ux + mxy * uy + mxz * uz;
    const T muy = mxy * ux + myy * uy + myz * uz;
    const T muz = mxz * ux + myz * uy + mzz * uz;
    const T s0 = a * (T(1) - K::C * uu) + K::A * (ux * bx + uy * by + uz * bz) +
                 K::B * (ux * mux + uy * muy + uz * muz);
    const T c2a = T(2) * K::C * a;
    const T vx = K::A * bx + T(2) * K::B * mux - c2a * ux;
    const T vy = K::A * by + T(2) * K::B * muy - c2a * uy;
    const T vz = K::A * bz + T(2) * K::B * muz - c2a * uz;
    const T k0 = omega * (s0 - (ux * vx + uy * vy + uz * vz));
    const T wx = omega * vx, wy = omega * vy, wz = omega * vz;
    const T om1 = T(1) - omega;
#pragma unroll
    for (int p = 0; p < L::Q; ++p) {
        T t = k0;
        add_signed(t, wx, L::c(p, 0));
        add_signed(t, wy, L::c(p, 1));
        add_signed(t, wz, L::c(p, 2));
        lam[p] = om1 * lam[p] + t;
    }
}

// d feq_q / d u_d at (rho0, u), for the handler terms.
template <class L, class T>
__device__ __forceinline__ T dfeq_du(int q, int d, T rho0, T cu, T ud)
{
    using K = AdjConst<T>;
    return T(rt_w<L>(q)) * rho0 * ((K::A + T(2) * K::B * cu) * T(rt_c<L>(q, d)) - T(2) * K::C * ud);
}

// Sums each moving-wall handler's gradient over the warp and adds it with one atomic per handler
// and warp (the lid of a cavity would otherwise send every link's atomics to the same three
// addresses). Every lane of the warp must call it.
__device__ __forceinline__ void warp_flush_wall(double* grad_wall, int hid, const double (&gw)[3])
{
    const unsigned full = 0xffffffffu;
    const int lane = static_cast<int>(threadIdx.x & 31);
    int mine = hid;
    for (;;) {
        const unsigned pending = __ballot_sync(full, mine >= 0);
        if (!pending) break;
        const int leader = __ffs(pending) - 1;
        const int target = __shfl_sync(full, mine, leader);
        double v[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] = mine == target ? gw[k] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) v[k] += __shfl_xor_sync(full, v[k], o);
        if (lane == leader)
#pragma unroll
            for (int k = 0; k < 3; ++k) atomicAdd(grad_wall + 3 * target + k, v[k]);
        if (mine == target) mine = -1;
    }
}

// Blocks per SM the FP32 adjoint step is compiled for (0: no bound; FP64 is never bounded). The
// kernel is latency-bound (on the 128x64x64 channel every pipe is below 11% busy with 20 of 64
// warps active), so more resident warps pay where they cost no spills: D3Q15 and D3Q19 at 9 blocks
// (56 registers; the channel's backward 52.2 against 56.0 us per step unbounded at 64). D3Q27
// spills at 9 and stays unbounded (68 registers). LBMG_ADJ_MINB sets every stencil in tuning
// builds.
template <class L, class T>
constexpr int adj_min_blocks()
{
#ifdef LBMG_ADJ_MINB
    return sizeof(T) == 4 ? LBMG_ADJ_MINB : 0;
#else
    return sizeof(T) == 4 && L::Q != 27 ? 9 : 0;
#endif
}

template <class L, class T>
__global__ void __launch_bounds__(kBlockX, adj_min_blocks<L, T>()) adjoint_step_kernel(const AdjParams<T> A)
{
    using K = AdjConst<T>;
    constexpr int Q = L::Q;
    grid_dep_wait();  // the previous adjoint step (or the kernel before it) has completed
    grid_dep_launch();
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = cidx(A.g, x, y, z);
    const uint8_t fl = x <= A.g.xl ? A.flag[i] : static_cast<uint8_t>(0xff);
    const bool active = is_fluid(fl);
    int wall_h = -1;               // moving-wall handler whose gradient this thread accumulates
    double gw[3] = {0.0, 0.0, 0.0};
    if (active) {
        const size_t PS = A.g.PS;
        const uint2 lw = fl != kFluidBulk ? A.link[i] : make_uint2(0u, kNoRecord);
        const uint32_t link = lw.x;  // bit q: x - c_q is a boundary cell
        // the links whose handler terms apply this step
        const uint32_t own = A.bc_terms ? link : 0u;
        T lam[Q];
        // transposed pull: x's f*_p became the pulled g_p of x + c_p. Non-fluid cells hold 0 in
        // every adjoint array (cleared once, never written), so no neighbour test is needed. For a
        // link q the pull of direction inv(q) meets such a cell; that slot reads x's own mu_q
        // instead, the quantity every handler term of q starts from (for no-slip, lam[inv q] += mu_q
        // is the whole term). Bulk cells have no wrapped neighbour either.
        if (fl != kFluidEdge) {  // no wrapped neighbour
            // one running pointer over the planes (block-uniform deltas), as the step's stores
            const int sy = A.g.XS, sz = A.g.XS * A.g.YS;
            const T* ptr = A.mu_in + i + (L::c(0, 0) + L::c(0, 1) * sy + L::c(0, 2) * sz);
#pragma unroll
            for (int p = 0; p < Q; ++p) {
                const int qo = Q - 1 - p;  // the link whose pull partner is direction p
                const long long self = static_cast<long long>(qo - p) * static_cast<long long>(PS) -
                                       (L::c(p, 0) + L::c(p, 1) * sy + L::c(p, 2) * sz);
                lam[p] = __ldcs(((own >> qo) & 1u) ? ptr + self : ptr);
                if (p + 1 < Q) {
                    const int d = (L::c(p + 1, 0) - L::c(p, 0)) + (L::c(p + 1, 1) - L::c(p, 1)) * sy +
                                  (L::c(p + 1, 2) - L::c(p, 2)) * sz;
                    ptr += static_cast<long long>(PS) + d;
                }
            }
        } else {
#pragma unroll
            for (int p = 0; p < Q; ++p) {
                const int qo = Q - 1 - p;
                size_t k;
                if ((own >> qo) & 1u) {
                    k = static_cast<size_t>(qo) * PS + i;
                } else {
                    int mx, my, mz;
                    nbr_xyz(A.g, x, y, z, L::c(p, 0), L::c(p, 1), L::c(p, 2), mx, my, mz);
                    k = static_cast<size_t>(p) * PS + cidx(A.g, mx, my, mz);
                }
                lam[p] = __ldcs(&A.mu_in[k]);
            }
        }
        T rho_s, jxs, jys, jzs;
        ld_rec4(A.rec + 4 * static_cast<size_t>(i), rho_s, jxs, jys, jzs);
        // links whose handler needs its table entry: every link of a kFluidEdge cell; of a
        // kFluidWall cell only those its LinkRecord lists (the others are no-slip, done above)
        uint32_t generic = own;
        if (fl == kFluidWall) generic = (lw.y != kNoRecord && A.ltab) ? A.ltab[lw.y].spec & own : 0u;
        if (generic) {
            T spread = 0;              // added to every direction (handlers that use sum f*)
            T sx = 0, sy = 0, sz = 0;  // outflow / pressure: added as c_p . s
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                if (!((generic >> q) & 1u)) continue;
                const int qb = L::Q - 1 - q;
                const T mu_q = lam[qb];  // read by the pull above; the pull term itself is 0
                int bx, by, bz;
                nbr_xyz(A.g, x, y, z, -L::c(q, 0), -L::c(q, 1), -L::c(q, 2), bx, by, bz);
                const uint8_t flb = A.flag[cidx(A.g, bx, by, bz)];
                if (flb < kFirstHandler) {  // no handler: no term
                    lam[qb] = T(0);
                    continue;
                }
                const int h = flb - kFirstHandler;
                const BcEntry& be = A.bc[h];
                switch (be.type) {
                case kNoSlip:  // B_q = f*_qb: lam[qb] += mu_q, already in place
                    break;
                case kMovingWall: {  // B_q = f*_qb + 2 w_q rho* (c_q . u_w) / cs2
                    const T cuw = T(L::c(q, 0)) * T(be.v[0]) + T(L::c(q, 1)) * T(be.v[1]) +
                                  T(L::c(q, 2)) * T(be.v[2]);
                    spread += mu_q * T(2) * T(L::w(q)) * cuw * K::A;
                    const double gcoef = static_cast<double>(mu_q * T(2) * T(L::w(q)) * rho_s * K::A);
                    if (wall_h < 0) wall_h = h;
                    if (h == wall_h) {
                        gw[0] += gcoef * L::c(q, 0);
                        gw[1] += gcoef * L::c(q, 1);
                        gw[2] += gcoef * L::c(q, 2);
                    } else {
                        atomicAdd(A.grad_wall + 3 * h + 0, gcoef * L::c(q, 0));
                        atomicAdd(A.grad_wall + 3 * h + 1, gcoef * L::c(q, 1));
                        atomicAdd(A.grad_wall + 3 * h + 2, gcoef * L::c(q, 2));
                    }
                    break;
                }
                case kInflow: {  // B_q = feq_q(rho0, u_in): no f* term
                    lam[qb] = T(0);
                    const size_t r = ref_idx(A.g, bx, by, bz);
                    const double* v = be.has_profile ? A.profile + 3 * r : be.v;
                    const T vx = T(v[0]), vy = T(v[1]), vz = T(v[2]);
                    const T cu = T(L::c(q, 0)) * vx + T(L::c(q, 1)) * vy + T(L::c(q, 2)) * vz;
                    const T r0 = T(be.rho);
                    atomicAdd(A.grad_inflow + 3 * r + 0, static_cast<double>(mu_q * dfeq_du<L, T>(q, 0, r0, cu, vx)));
                    atomicAdd(A.grad_inflow + 3 * r + 1, static_cast<double>(mu_q * dfeq_du<L, T>(q, 1, r0, cu, vy)));
                    atomicAdd(A.grad_inflow + 3 * r + 2, static_cast<double>(mu_q * dfeq_du<L, T>(q, 2, r0, cu, vz)));
                    break;
                }
                case kOutflow:
                case kPressure: {
                    // B_q = feq_q(r0, u) + feq_qb(r0, u) - f*_qb with u = j*/r0:
                    // dB_q/df*_p = (D . c_p)/r0 - delta(p, qb), D_d = w_q r0 (4 B cu c_qd - 4 C u_d)
                    const T r0 = T(be.rho);
                    const T ux = jxs / r0, uy = jys / r0, uz = jzs / r0;
                    const T cu = T(L::c(q, 0)) * ux + T(L::c(q, 1)) * uy + T(L::c(q, 2)) * uz;
                    const T wr = T(L::w(q)) * r0;
                    const T dx = wr * (T(4) * K::B * cu * T(L::c(q, 0)) - T(4) * K::C * ux);
                    const T dy = wr * (T(4) * K::B * cu * T(L::c(q, 1)) - T(4) * K::C * uy);
                    const T dz = wr * (T(4) * K::B * cu * T(L::c(q, 2)) - T(4) * K::C * uz);
                    lam[qb] = -mu_q;
                    sx += mu_q * dx / r0;
                    sy += mu_q * dy / r0;
                    sz += mu_q * dz / r0;
                    break;
                }
                default:
                    lam[qb] = T(0);
                    break;
                }
            }
#pragma unroll
            for (int p = 0; p < Q; ++p)
                lam[p] += spread + T(L::c(p, 0)) * sx + T(L::c(p, 1)) * sy + T(L::c(p, 2)) * sz;
        }
        if (A.write_mu) {
            bgk_adjoint<L, T>(lam, rho_s, jxs, jys, jzs, A.omega);
            T* out = A.mu_out + i;
#pragma unroll
            for (int p = 0; p < Q; ++p) {
                __stcs(out, lam[p]);
                out += PS;
            }
        }
    }
    if (A.bc_terms) warp_flush_wall(A.grad_wall, wall_h, gw);
}

// mu_T = J^T lambda_T with lambda_T = dJ/df*_T of J = sum_{x in box} rho |u|^2 / 2, i.e.
// lambda_T(x)_p = u . c_p - |u|^2 / 2 inside the box (u of the final state), 0 outside.
template <class L, class T>
__global__ void __launch_bounds__(kBlockX)
    adjoint_terminal_kernel(const uint8_t* flag, Geom g, T omega, const T* rec, Box box, T* mu_out)
{
    constexpr int Q = L::Q;
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = cidx(g, x, y, z);
    if (!is_fluid(flag[i])) return;
    T rho, jx, jy, jz;
    ld_rec4(rec + 4 * static_cast<size_t>(i), rho, jx, jy, jz);
    const bool in = x >= box.x0 && x <= box.x1 && y >= box.y0 && y <= box.y1 && z >= box.z0 && z <= box.z1;
    const T ux = jx / rho, uy = jy / rho, uz = jz / rho;
    const T half_uu = T(0.5) * (ux * ux + uy * uy + uz * uz);
    T lam[Q];
#pragma unroll
    for (int p = 0; p < Q; ++p)
        lam[p] = in ? T(L::c(p, 0)) * ux + T(L::c(p, 1)) * uy + T(L::c(p, 2)) * uz - half_uu : T(0);
    bgk_adjoint<L, T>(lam, rho, jx, jy, jz, omega);
#pragma unroll
    for (int p = 0; p < Q; ++p) mu_out[static_cast<size_t>(p) * g.PS + i] = lam[p];
}

// Kinetic energy sum_{x in box, fluid} rho |u|^2 / 2 of the post-collision state, FP64; one
// partial per block (fixed grid), summed in order by reduce_final_kernel.
template <class L, class S>
__global__ void __launch_bounds__(kReduceThreads)
    objective_ke_kernel(const S* pop, const uint8_t* flag, Geom g, int odd, Box box, double* partials)
{
    double acc = 0.0;
    const int bx = box.x1 - box.x0 + 1, by = box.y1 - box.y0 + 1, bz = box.z1 - box.z0 + 1;
    const size_t n = static_cast<size_t>(bx) * by * bz;
    for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int x = box.x0 + static_cast<int>(k % bx);
        const int y = box.y0 + static_cast<int>((k / bx) % by);
        const int z = box.z0 + static_cast<int>(k / (static_cast<size_t>(bx) * by));
        const int i = cidx(g, x, y, z);
        if (!is_fluid(flag[i])) continue;
        double m[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int p = 0; p < L::Q; ++p) {
            const double f = to_f64<L, S>(load_post<L, S>(pop, flag, g, x, y, z, i, p, odd != 0), p);
            m[0] += f;
            m[1] += L::c(p, 0) * f;
            m[2] += L::c(p, 1) * f;
            m[3] += L::c(p, 2) * f;
        }
        acc += 0.5 * (m[1] * m[1] + m[2] * m[2] + m[3] * m[3]) / m[0];
    }
    __shared__ double red[kReduceThreads / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < kReduceThreads / 32; ++w) v += red[w];
        partials[4 * blockIdx.x] = v;
        partials[4 * blockIdx.x + 1] = 0.0;
        partials[4 * blockIdx.x + 2] = 0.0;
        partials[4 * blockIdx.x + 3] = 0.0;
    }
}

}  // namespace lbmg
