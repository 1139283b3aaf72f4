// Internal state of one lattice Boltzmann domain on the device, shared by the host C-ABI layer
// (capi.cu) and the per-precision kernel translation units (step_*.cu).
//
// HBM layout
//   pop   : Q planes of PS elements each (structure of arrays). Cell (x, y, z), ghost layer
//           included, sits at column kXOff + x of row (y, z): index kXOff + x + XS*(y + YS*z),
//           XS = round_up(xl + 2, 32), YS = yl + 2. Interior rows start at column 32, so every
//           warp's 32 consecutive x cells begin on a 32-element boundary. The ghost cell
//           x = xl + 1 may spill into the next row's unused columns 0..30.
//           Planes are PS = round_up(XS*YS*ZS + 512, 64) elements apart; the slack after the
//           last row absorbs the widened row copies of the row kernel.
//   flag  : one byte per cell, same indexing (see CellFlag).
//   link  : one 32-bit word per cell, same indexing (fluid cells only, see classify_kernel).
//   State after k steps, in place (AA pattern): for an interior fluid cell x and direction p
//   with neighbour m = x + c_p,
//     k even : f*_p(x) is at plane inv(p), cell x when m is fluid; at plane p, cell m otherwise
//     k odd  : f*_p(x) is at plane p, cell m
//   and for every direction q whose upstream neighbour x - c_q is not fluid, plane q at cell x
//   holds what that neighbour's boundary handler wrote for x (the value x pulls next step).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace lbmg {

// Column of the ghost cell x = 0 inside a row.
constexpr int kXOff = 31;
// Threads per block along x for the cell-parallel kernels.
constexpr int kBlockX = 128;

// Per-cell byte flag.
enum CellFlag : uint8_t {
    kFluidBulk = 0,   // fluid; every neighbour is fluid and none wraps around a periodic axis
    kFluidEdge = 1,   // fluid; at least one neighbour is not fluid or wraps
    kGhostFluid = 2,  // ghost-layer cell without a boundary condition (reference: a fluid cell
                      // that collides in place but never streams, domain.hpp:143-166), or a
                      // ghost cell of a periodic axis (never referenced)
    kFirstHandler = 3 // kFirstHandler + h - 1 : non-fluid cell bound to handler h (1-based)
};
constexpr int kMaxHandlers = 250;
// Accumulator buckets of the step monitor (atomics of different warps spread over them).
constexpr int kMonBuckets = 256;

// Boundary-handler types (values match LBM_NOSLIP ... LBM_PRESSURE in lbm_gb300.h).
enum BcType : int {
    kNoSlip = 1, kMovingWall = 2, kFreeSlip = 3, kOutflow = 4, kInflow = 5, kPressure = 6
};

struct BcEntry {
    int type;
    int has_profile;  // inflow only: velocity per cell from DomainDev::profile
    double v[3];      // wall / inflow velocity
    double rho;       // rho-ref (inflow, outflow) or rho-in (pressure)
};

// An inclusive box of interior cells (the objective region of the adjoint).
struct Box {
    int x0, x1, y0, y1, z0, z1;
};

struct Geom {
    int xl, yl, zl;
    int XS, YS, ZS;  // row stride (elements), rows per plane slice (yl+2), slices (zl+2)
    int per;         // periodic axes: bit 0 = x, bit 1 = y, bit 2 = z
    size_t PS;       // plane stride (elements)
};

// Device-side view handed to the kernel launchers.
struct DomainDev {
    Geom g;
    int q;
    int precision;
    double tau;
    void* pop;                 // Q * PS storage elements
    uint8_t* flag;             // PS bytes
    const BcEntry* bc;         // kMaxHandlers entries
    const double* profile;     // 3 doubles per cell in reference cell order, or nullptr
    // Ghost-fluid side pass: cells in the ghost layer without a handler that have at least one
    // interior fluid neighbour (or feed a free-slip link). Two FP64 copies of their populations
    // (the reference's two fields), n_gf entries each.
    const int* gf_xyz;         // x, y, z per ghost-fluid cell
    double* gf_pop;            // [2][n_gf][Q]
    int n_gf;
    // Free-slip side pass: one entry per (boundary cell, direction) link that a free-slip
    // handler writes (see the free-slip link note below).
    const int4* fs_link;
    int n_fs;
    // Per interior fluid cell: which pull neighbours are not fluid (see classify_kernel).
    uint32_t* link;
    // kFluidEdge cells as layout indices in increasing order: updated by the edge blocks of the
    // step kernel; all other fluid cells by its row blocks.
    const int* edge;
    int n_edge;
    // Device error word: set to 1 by a kernel whose bounded wait gave up.
    int* err;
    // Step monitor accumulators (kMonBuckets x 4 doubles, zero between steps).
    double* mon;
};

// A free-slip link: after a step, plane `q` at fluid cell `dst` receives the post-collision
// population `qs` of source cell `src` (boundary.hpp:79-115). src_kind 0: interior fluid cell;
// 1: ghost-fluid cell, src then indexes the ghost-fluid list.
// Packed as int4 {dst, q | (qs << 8) | (src_kind << 16), src, src_m} where src_m is the cell
// index of src + c_qs (used to locate the population in the AA layout).

}  // namespace lbmg
