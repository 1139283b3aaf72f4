// Kernels around the time step: initialisation, cell classification, conversion between the
// in-place device layout and the reference's AoS population field, moments, the FP64
// conservation reduction, and the two side passes (ghost-fluid cells, free-slip links).
#pragma once

#include "kernels.cuh"

namespace lbmg {

// Every plane q holds w_q (FP64 store) or 0 (shifted stores): the reference's initial state
// (cell.hpp:8-15) in any layout parity and for any geometry, boundary slots included.
template <class L, class S>
__global__ void init_kernel(S* pop, size_t PS)
{
    const size_t n = static_cast<size_t>(L::Q) * PS;
    for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int q = static_cast<int>(k / PS);
        Store<S>::st(pop + k, from_f64<L, S>(L::w(q), q));
    }
}

// Interior fluid cells: kFluidEdge when some neighbour is not fluid or lies across a periodic
// wrap, else kFluidBulk; and their link word (bit q: the pull neighbour x - c_q is not fluid).
// The lattice is symmetric, so the pull neighbours x - c_q are also all the push neighbours.
template <class L>
// special_ok (shifted storage): links to moving-wall, inflow, outflow and pressure cells (at most
// kMaxRecordValues moving-wall and inflow links, one outlet density) keep a cell in the row blocks,
// served by its LinkRecord.
__global__ void classify_kernel(uint8_t* flag, uint2* link, const BcEntry* bc, Geom g, bool special_ok)
{
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = cidx(g, x, y, z);
    if (!is_fluid(flag[i])) return;
    bool edge = false;  // some neighbour wraps or needs the edge path's handling
    uint32_t m = 0;
    int values = 0;      // moving-wall and inflow links (one LinkRecord value each)
    double r0 = -1.0;    // reference density of the outflow / pressure links
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        const int ax = x - L::c(q, 0), ay = y - L::c(q, 1), az = z - L::c(q, 2);
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, -L::c(q, 0), -L::c(q, 1), -L::c(q, 2), nx, ny, nz);
        if (nx != ax || ny != ay || nz != az) edge = true;
        // flags of fluid cells only move among the fluid values here, so this read of a
        // neighbour's flag sees the same fluid / non-fluid answer whatever the timing
        const uint8_t fn = flag[cidx(g, nx, ny, nz)];
        if (!is_fluid(fn)) {
            m |= 1u << q;
            const int t = fn < kFirstHandler ? -1 : bc[fn - kFirstHandler].type;
            if (t == kNoSlip) {
            } else if (special_ok && (t == kMovingWall || t == kInflow)) {
                ++values;
            } else if (special_ok && (t == kOutflow || t == kPressure)) {
                const double r = bc[fn - kFirstHandler].rho;
                if (r0 >= 0.0 && r != r0) edge = true;  // one outlet density per cell
                r0 = r;
            } else {
                edge = true;
            }
        }
    }
    if (values > kMaxRecordValues) edge = true;
    flag[i] = edge ? kFluidEdge : (m ? kFluidWall : kFluidBulk);
    link[i] = make_uint2(m, kNoRecord);
}

// Per row segment of the step kernel (kRowCells cells of one row from x0; segment index
// sx + nseg_x * ((y - 1) + yl * (z - 1)), the row blocks' order): bit w set when the segment's warp
// w covers kFluidBulk cells only, all inside the row. Row blocks skip the per-cell flag, link and
// handler work of such a warp. Grid (nseg_x, yl, zl), kRowCells threads.
static __global__ void __launch_bounds__(kRowCells) warp_mask_kernel(const uint8_t* flag, Geom g, int nseg_x,
                                                                     uint8_t* wmask)
{
    __shared__ unsigned bits;
    if (threadIdx.x == 0) bits = 0u;
    __syncthreads();
    const int sx = static_cast<int>(blockIdx.x);
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int x = 1 + sx * kRowCells + static_cast<int>(threadIdx.x);
    const bool bulk = x <= g.xl && flag[cidx(g, x, y, z)] == kFluidBulk;
    if (__all_sync(0xffffffffu, bulk) && (threadIdx.x & 31u) == 0u) atomicOr(&bits, 1u << (threadIdx.x >> 5));
    __syncthreads();
    if (threadIdx.x == 0)
        wmask[sx + static_cast<size_t>(nseg_x) * ((y - 1) + static_cast<size_t>(g.yl) * (z - 1))] =
            static_cast<uint8_t>(bits);
}

// LinkRecord of every kFluidWall cell with links to handlers other than no-slip (shifted
// storage). Rows are handed out by an atomic counter; with capacity 0 it only counts them.
template <class L>
__global__ void link_table_kernel(const uint8_t* flag, uint2* link, const BcEntry* bc, const double* profile,
                                  Geom g, LinkRecord* ltab, int* counter, int capacity)
{
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = cidx(g, x, y, z);
    if (flag[i] != kFluidWall) return;
    const uint32_t lk = link[i].x;
    LinkRecord r{};
    int k = 0;
    for (int q = 0; q < L::Q; ++q) {
        if (!((lk >> q) & 1u)) continue;
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, -rt_c<L>(q, 0), -rt_c<L>(q, 1), -rt_c<L>(q, 2), nx, ny, nz);
        const BcEntry& be = bc[flag[cidx(g, nx, ny, nz)] - kFirstHandler];
        if (be.type == kNoSlip) continue;
        r.spec |= 1u << q;
        if (be.type == kOutflow || be.type == kPressure) {
            r.r0 = static_cast<float>(be.rho);
            r.ir0 = 1.f / r.r0;
            continue;
        }
        if (k >= kMaxRecordValues) continue;  // classify sent such cells to the edge blocks
        if (be.type == kMovingWall) {
            const float cu = rt_c<L>(q, 0) * static_cast<float>(be.v[0]) + rt_c<L>(q, 1) * static_cast<float>(be.v[1]) +
                             rt_c<L>(q, 2) * static_cast<float>(be.v[2]);
            r.wall |= 1u << q;
            r.c[k++] = 2.f * static_cast<float>(rt_w<L>(q)) * cu * kA;
        } else {
            const double* v = be.has_profile ? profile + 3 * ref_idx(g, nx, ny, nz) : be.v;
            const float rr = static_cast<float>(be.rho);
            const float ux = static_cast<float>(v[0]), uy = static_cast<float>(v[1]), uz = static_cast<float>(v[2]);
            r.inflow |= 1u << q;
            r.c[k++] = seq_shifted<L>(q, rr - 1.f, rr, ux, uy, uz, (ux * ux + uy * uy + uz * uz) * kC);
        }
    }
    if (!r.spec) return;
    const int row = atomicAdd(counter, 1);
    if (row < capacity) {
        link[i].y = static_cast<uint32_t>(row);
        ltab[row] = r;
    }
}

// Device layout -> AoS FP64 field over all cells (reference cell order).
template <class L, class S>
__global__ void gather_kernel(const S* pop, const uint8_t* flag, Geom g, int odd, double* out)
{
    const size_t ng = static_cast<size_t>(g.xl + 2) * (g.yl + 2) * (g.zl + 2);
    for (size_t r = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; r < ng;
         r += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int x = static_cast<int>(r % (g.xl + 2));
        const int y = static_cast<int>((r / (g.xl + 2)) % (g.yl + 2));
        const int z = static_cast<int>(r / (static_cast<size_t>(g.xl + 2) * (g.yl + 2)));
        double f[L::Q];
        load_cell_f64<L, S>(pop, flag, g, x, y, z, odd != 0, f);
#pragma unroll
        for (int q = 0; q < L::Q; ++q) out[r * L::Q + q] = f[q];
    }
}

// AoS FP64 field (reference order) -> device layout with the given parity. One thread per
// interior fluid cell writes its own post-collision slots and the boundary slots it pulls from.
template <class L, class S>
__global__ void scatter_kernel(S* pop, const uint8_t* flag, Geom g, int odd, const double* in)
{
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    const int i = cidx(g, x, y, z);
    if (!is_fluid(flag[i])) return;
    const size_t r = ref_idx(g, x, y, z);
#pragma unroll
    for (int p = 0; p < L::Q; ++p) {
        const auto v = from_f64<L, S>(in[r * L::Q + p], p);
        if (!odd) {
            Store<S>::st(pop + static_cast<size_t>(inv<L>(p)) * g.PS + i, v);
        } else {
            int mx, my, mz;
            nbr_xyz(g, x, y, z, L::c(p, 0), L::c(p, 1), L::c(p, 2), mx, my, mz);
            Store<S>::st(pop + static_cast<size_t>(p) * g.PS + cidx(g, mx, my, mz), v);
        }
    }
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, -L::c(q, 0), -L::c(q, 1), -L::c(q, 2), nx, ny, nz);
        const int n = cidx(g, nx, ny, nz);
        if (is_fluid(flag[n])) continue;
        const auto v = from_f64<L, S>(in[ref_idx(g, nx, ny, nz) * L::Q + q], q);
        if (odd)
            Store<S>::st(pop + static_cast<size_t>(q) * g.PS + i, v);
        else
            Store<S>::st(pop + static_cast<size_t>(inv<L>(q)) * g.PS + n, v);
    }
}

// Stores the value that non-fluid cell b = (bx, by, bz) hands to its fluid neighbour n = b + c_q
// (layout index n), where n pulls it next step: after an odd step plane q at n, after an even
// step plane inv(q) at b.
template <class L, class S>
__device__ __forceinline__ void store_slot(S* pop, const Geom& g, int odd, int n, int bx, int by, int bz, int q,
                                           typename Store<S>::C v)
{
    if (odd)
        Store<S>::st(pop + static_cast<size_t>(q) * g.PS + n, v);
    else
        Store<S>::st(pop + static_cast<size_t>(L::Q - 1 - q) * g.PS + cidx(g, bx, by, bz), v);
}

// Cell (x, y, z) of row r of the reference's cell order (domain.hpp:60-64).
__device__ __forceinline__ void ref_xyz(const Geom& g, size_t r, int& x, int& y, int& z)
{
    const size_t nx = static_cast<size_t>(g.xl + 2), nxy = nx * static_cast<size_t>(g.yl + 2);
    z = static_cast<int>(r / nxy);
    const size_t t = r - static_cast<size_t>(z) * nxy;
    y = static_cast<int>(t / nx);
    x = static_cast<int>(t - static_cast<size_t>(y) * nx);
}

__device__ __forceinline__ bool on_periodic_ghost(const Geom& g, int x, int y, int z)
{
    return ((g.per & 1) && (x == 0 || x == g.xl + 1)) || ((g.per & 2) && (y == 0 || y == g.yl + 1)) ||
           ((g.per & 4) && (z == 0 || z == g.zl + 1));
}

// Rows [r0, r1) of the AoS FP64 field (reference cell order) from the device layout, row r into
// out[(r - r0) * Q ..]: one chunk of a read-back through the handle's staging buffers. Ghost-fluid
// cells come out as w_q; the host writes their side copies over them.
template <class L, class S>
__global__ void gather_range_kernel(const S* pop, const uint8_t* flag, Geom g, int odd, size_t r0, size_t r1,
                                    double* out)
{
    for (size_t r = r0 + blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; r < r1;
         r += static_cast<size_t>(gridDim.x) * blockDim.x) {
        int x, y, z;
        ref_xyz(g, r, x, y, z);
        double f[L::Q];
        load_cell_f64<L, S>(pop, flag, g, x, y, z, odd != 0, f);
        double* o = out + (r - r0) * L::Q;
#pragma unroll
        for (int q = 0; q < L::Q; ++q) o[q] = f[q];
    }
}

// Rows [r0, r1) of the AoS FP64 field (row r at in[(r - r0) * Q ..]) into the device layout with
// the given parity: one chunk of an upload. An interior fluid cell writes its own post-collision
// slots; a handler cell writes, for each direction q whose neighbour b + c_q is an interior fluid
// cell, the slot that neighbour pulls from it (the value its handler wrote in the reference's
// collide_field). Ghost-fluid cells are written from their side copies afterwards
// (ghost_fluid_slots_kernel); cells on the ghost planes of periodic axes are never read.
template <class L, class S>
__global__ void scatter_range_kernel(S* pop, const uint8_t* flag, Geom g, int odd, size_t r0, size_t r1,
                                     const double* in)
{
    for (size_t r = r0 + blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; r < r1;
         r += static_cast<size_t>(gridDim.x) * blockDim.x) {
        int x, y, z;
        ref_xyz(g, r, x, y, z);
        const int i = cidx(g, x, y, z);
        const uint8_t fl = flag[i];
        const double* row = in + (r - r0) * L::Q;
        if (is_fluid(fl) && interior(g, x, y, z)) {
#pragma unroll
            for (int p = 0; p < L::Q; ++p) {
                const auto v = from_f64<L, S>(row[p], p);
                if (!odd) {
                    Store<S>::st(pop + static_cast<size_t>(inv<L>(p)) * g.PS + i, v);
                } else {
                    int mx, my, mz;
                    nbr_xyz(g, x, y, z, L::c(p, 0), L::c(p, 1), L::c(p, 2), mx, my, mz);
                    Store<S>::st(pop + static_cast<size_t>(p) * g.PS + cidx(g, mx, my, mz), v);
                }
            }
        } else if (fl >= kFirstHandler && !on_periodic_ghost(g, x, y, z)) {
#pragma unroll
            for (int q = 0; q < L::Q; ++q) {
                int nx, ny, nz;
                nbr_xyz(g, x, y, z, L::c(q, 0), L::c(q, 1), L::c(q, 2), nx, ny, nz);
                if (!interior(g, nx, ny, nz)) continue;
                const int n = cidx(g, nx, ny, nz);
                if (!is_fluid(flag[n])) continue;
                store_slot<L, S>(pop, g, odd, n, x, y, z, q, from_f64<L, S>(row[q], q));
            }
        }
    }
}

// Density and velocity of the interior cells [n0, n1) of the interior order (vtk.hpp:62-73 ->
// collision.hpp:6-31), FP64: rho_out[n - n0] and u_out[3 (n - n0) ..]; one chunk of lbm_moments.
template <class L, class S>
__global__ void moments_range_kernel(const S* pop, const uint8_t* flag, Geom g, int odd, size_t n0, size_t n1,
                                     double* rho_out, double* u_out)
{
    const size_t nx = static_cast<size_t>(g.xl), nxy = nx * static_cast<size_t>(g.yl);
    for (size_t n = n0 + blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; n < n1;
         n += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int z = static_cast<int>(n / nxy);
        const size_t t = n - static_cast<size_t>(z) * nxy;
        const int y = static_cast<int>(t / nx);
        const int x = static_cast<int>(t - static_cast<size_t>(y) * nx);
        double f[L::Q];
        load_cell_f64<L, S>(pop, flag, g, x + 1, y + 1, z + 1, odd != 0, f);
        const double rho = density_exact<L>(f);
        const size_t o = n - n0;
        rho_out[o] = rho;
        if (u_out) {
            u_out[3 * o + 0] = momentum_exact<L>(f, 0) / rho;
            u_out[3 * o + 1] = momentum_exact<L>(f, 1) / rho;
            u_out[3 * o + 2] = momentum_exact<L>(f, 2) / rho;
        }
    }
}

// Density and velocity of interior cells (vtk.hpp:62-73 -> collision.hpp:6-31), FP64, written
// as rho[n] and u[3n..3n+2] in interior order.
template <class L, class S>
__global__ void moments_kernel(const S* pop, const uint8_t* flag, Geom g, int odd,
                               double* rho_out, double* u_out)
{
    const int x = 1 + static_cast<int>(blockIdx.x) * kBlockX + static_cast<int>(threadIdx.x);
    if (x > g.xl) return;
    const int y = 1 + static_cast<int>(blockIdx.y), z = 1 + static_cast<int>(blockIdx.z);
    double f[L::Q];
    load_cell_f64<L, S>(pop, flag, g, x, y, z, odd != 0, f);
    const double rho = density_exact<L>(f);
    const size_t n = static_cast<size_t>(x - 1) +
                     static_cast<size_t>(g.xl) * (static_cast<size_t>(y - 1) +
                                                  static_cast<size_t>(g.yl) * (z - 1));
    rho_out[n] = rho;
    if (u_out) {
        u_out[3 * n + 0] = momentum_exact<L>(f, 0) / rho;
        u_out[3 * n + 1] = momentum_exact<L>(f, 1) / rho;
        u_out[3 * n + 2] = momentum_exact<L>(f, 2) / rho;
    }
}

// FP64 totals {sum rho, sum j} over interior fluid cells. Each block writes one partial into
// `partials` (4 doubles per block); reduce_final_kernel adds them in block order, so the result
// does not depend on scheduling.
constexpr int kReduceThreads = 256;

template <class L, class S>
__global__ void __launch_bounds__(kReduceThreads)
    reduce_kernel(const S* pop, const uint8_t* flag, Geom g, int odd, double* partials)
{
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const size_t n = static_cast<size_t>(g.xl) * g.yl * g.zl;
    for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int x = 1 + static_cast<int>(k % g.xl);
        const int y = 1 + static_cast<int>((k / g.xl) % g.yl);
        const int z = 1 + static_cast<int>(k / (static_cast<size_t>(g.xl) * g.yl));
        const int i = cidx(g, x, y, z);
        if (!is_fluid(flag[i])) continue;
#pragma unroll
        for (int p = 0; p < L::Q; ++p) {
            const double f = to_f64<L, S>(load_post<L, S>(pop, flag, g, x, y, z, i, p, odd != 0), p);
            acc[0] += f;
            acc[1] += L::c(p, 0) * f;
            acc[2] += L::c(p, 1) * f;
            acc[3] += L::c(p, 2) * f;
        }
    }
    __shared__ double red[4][kReduceThreads / 32];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < kReduceThreads / 32; ++w) v += red[threadIdx.x][w];
        partials[4 * blockIdx.x + threadIdx.x] = v;
    }
}

static __global__ void reduce_final_kernel(const double* partials, int nblocks, double* out)
{
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int b = 0; b < nblocks; ++b) v += partials[4 * b + threadIdx.x];
        out[threadIdx.x] = v;
    }
}

// ------------------------------------------------------------------------------------------
// Side pass 1: ghost-layer cells without a handler. The reference treats them as fluid cells
// that never stream (domain.hpp:115-141) but collide in place every step (domain.hpp:143-153),
// each of its two fields on its own: the copy in the field that is collide_field after step t
// is collided at step t. Interior fluid cells pull from them. Copy (t mod 2) is collided after
// step t and written into the boundary slots of the neighbours, which pull it at step t + 1.
// ------------------------------------------------------------------------------------------
template <class L, class S>
__global__ void ghost_fluid_kernel(S* pop, const uint8_t* flag, Geom g, DivRN tau,
                                   const int* gf_xyz, double* gf_pop, int n_gf, int copy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_gf) return;
    double* c = gf_pop + (static_cast<size_t>(copy) * n_gf + j) * L::Q;
    double f[L::Q];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) f[q] = c[q];
    double m[4];
    collide_exact<L>(f, tau, m);
    const int x = gf_xyz[3 * j], y = gf_xyz[3 * j + 1], z = gf_xyz[3 * j + 2];
#pragma unroll
    for (int q = 0; q < L::Q; ++q) {
        c[q] = f[q];
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, L::c(q, 0), L::c(q, 1), L::c(q, 2), nx, ny, nz);
        if (!interior(g, nx, ny, nz)) continue;
        const int n = cidx(g, nx, ny, nz);
        if (is_fluid(flag[n])) store_slot<L, S>(pop, g, copy, n, x, y, z, q, from_f64<L, S>(f[q], q));
    }
}

// Ghost-fluid copies from an AoS FP64 field (lbm_set_populations) and back (get).
template <class L>
__global__ void ghost_fluid_io_kernel(Geom g, const int* gf_xyz, double* gf_pop, int n_gf,
                                      int copy, double* aos, int to_aos)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_gf) return;
    double* c = gf_pop + (static_cast<size_t>(copy) * n_gf + j) * L::Q;
    const size_t r = ref_idx(g, gf_xyz[3 * j], gf_xyz[3 * j + 1], gf_xyz[3 * j + 2]);
    for (int q = 0; q < L::Q; ++q) {
        if (to_aos) aos[r * L::Q + q] = c[q];
        else c[q] = aos[r * L::Q + q];
    }
}

// Ghost-fluid copies written into the neighbours' boundary slots (after a scatter).
template <class L, class S>
__global__ void ghost_fluid_slots_kernel(S* pop, const uint8_t* flag, Geom g, const int* gf_xyz,
                                         const double* gf_pop, int n_gf, int copy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_gf) return;
    const double* c = gf_pop + (static_cast<size_t>(copy) * n_gf + j) * L::Q;
    const int x = gf_xyz[3 * j], y = gf_xyz[3 * j + 1], z = gf_xyz[3 * j + 2];
    for (int q = 0; q < L::Q; ++q) {
        int nx, ny, nz;
        nbr_xyz(g, x, y, z, L::c(q, 0), L::c(q, 1), L::c(q, 2), nx, ny, nz);
        if (!interior(g, nx, ny, nz)) continue;
        const int n = cidx(g, nx, ny, nz);
        if (is_fluid(flag[n])) store_slot<L, S>(pop, g, copy, n, x, y, z, q, from_f64<L, S>(c[q], q));
    }
}

// ------------------------------------------------------------------------------------------
// Side pass 2: free-slip links (boundary.hpp:79-115). The handler copies, for each direction q
// that faces an interior fluid cell, a mirrored post-collision population of another fluid
// cell; which cell and which direction is fixed by the geometry and precomputed on the host.
// Link = int4 {dst, q | qs << 8 | kind << 16, src, src_m}: plane q at cell dst receives
// population qs of source src (kind 0: interior fluid cell whose neighbour along c_qs is src_m;
// kind 1: ghost-fluid cell number src).
// ------------------------------------------------------------------------------------------
template <class L, class S>
__global__ void free_slip_kernel(S* pop, const uint8_t* flag, Geom g, const int4* links, int n,
                                 int odd, const double* gf_pop, int n_gf, int copy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int4 l = links[j];
    const int q = l.y & 0xff, qs = (l.y >> 8) & 0xff, kind = (l.y >> 16) & 0xff;
    typename Store<S>::C v;
    if (kind == 1) {
        v = from_f64<L, S>(gf_pop[(static_cast<size_t>(copy) * n_gf + l.z) * L::Q + qs], qs);
    } else if (!odd) {
        v = Store<S>::ld(pop + static_cast<size_t>(L::Q - 1 - qs) * g.PS + l.z);
    } else {
        v = Store<S>::ld(pop + static_cast<size_t>(qs) * g.PS + l.w);
    }
    // the free-slip cell b = dst - c_q
    const int r = l.x - kXOff;
    int bx, by, bz;
    nbr_xyz(g, r % g.XS, (r / g.XS) % g.YS, r / (g.XS * g.YS), -rt_c<L>(q, 0), -rt_c<L>(q, 1), -rt_c<L>(q, 2), bx, by, bz);
    store_slot<L, S>(pop, g, odd, l.x, bx, by, bz, q, v);
}

}  // namespace lbmg
