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
//     k even : f*_p(x) is at plane inv(p), cell x
//     k odd  : f*_p(x) is at plane p, cell m
//   A non-fluid cell b keeps the value its boundary handler wrote for the fluid cell n = b + c_q
//   (the population n pulls in direction q next step) where a fluid cell would keep its own
//   outgoing population q: k even at plane inv(q), cell b; k odd at plane q, cell n. So every
//   cell pulls the same way from fluid and non-fluid neighbours.
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
    kFluidEdge = 1,   // fluid; some neighbour wraps, or is non-fluid and not a no-slip cell
    kFluidWall = 2,   // fluid; no neighbour wraps, some are no-slip cells, all others are fluid
    kGhostFluid = 3,  // ghost-layer cell without a boundary condition (reference: a fluid cell
                      // that collides in place but never streams, domain.hpp:143-166), or a
                      // ghost cell of a periodic axis (never referenced)
    kFirstHandler = 4 // kFirstHandler + h - 1 : non-fluid cell bound to handler h (1-based)
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

// Handler record of a kFluidWall cell whose links include handlers other than no-slip
// (shifted storage only); bit q of a mask = the link from x - c_q. `spec`: every such link;
// `wall`: moving-wall links; `inflow`: inflow links; the rest of `spec` are outflow / pressure
// links, all with the reference density r0 (ir0 = 1 / r0). c[k], over the wall and inflow links
// in increasing q: moving wall 2 w_q (c_q . u_w) / cs2 (added times the cell's density to the
// bounce-back value), inflow the shifted equilibrium value itself.
constexpr int kMaxRecordValues = 11;
struct __align__(16) LinkRecord {
    uint32_t spec;
    uint32_t wall;
    uint32_t inflow;
    float r0;
    float ir0;
    float c[kMaxRecordValues];
};
constexpr uint32_t kNoRecord = 0xffffffffu;
static_assert(sizeof(LinkRecord) == 64, "LinkRecord is 16 words");

// Division of 32-bit unsigned integers by an invariant divisor d >= 1 through a multiply-high
// (Granlund and Montgomery, "Division by invariant integers using multiplication", PLDI 1994,
// round-up variant): with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> l for every 32-bit n (the sum taken in 64 bits).
struct FastDiv {
    uint32_t d, m, l;
};
inline FastDiv make_fastdiv(uint32_t d)
{
    FastDiv f{d, 0u, 0u};
    if (d > 1) {
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;
        f.l = l;
        f.m = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    return f;
}
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t fast_div(uint32_t n, const FastDiv& f)
{
    return static_cast<uint32_t>((static_cast<uint64_t>(__umulhi(n, f.m)) + n) >> f.l);
}
#endif

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
    // Per interior fluid cell: x = which pull neighbours are not fluid (see classify_kernel);
    // y = the cell's LinkRecord row, or kNoRecord.
    uint2* link;
    // kFluidEdge cells as layout indices in increasing order: updated by the edge blocks of the
    // step kernel; all other fluid cells by its row blocks.
    const int* edge;
    int n_edge;
    const LinkRecord* ltab;  // rows named by link[i].y
    // One byte per row segment of the step kernel: bit w = the segment's warp w holds only
    // kFluidBulk cells (see warp_mask_kernel).
    const uint8_t* wmask;
    // 1 when some cell is bound to a boundary handler (then fluid cells may have handler links)
    int links;
    // Device error word: set to 1 by a kernel whose bounded wait gave up.
    int* err;
    // Step monitor accumulators: two sets of kMonBuckets x 4 doubles, used by alternate monitored
    // steps (each set is zero while unused).
    double* mon;
};

// A free-slip link: after a step, plane `q` at fluid cell `dst` receives the post-collision
// population `qs` of source cell `src` (boundary.hpp:79-115). src_kind 0: interior fluid cell;
// 1: ghost-fluid cell, src then indexes the ghost-fluid list.
// Packed as int4 {dst, q | (qs << 8) | (src_kind << 16), src, src_m} where src_m is the cell
// index of src + c_qs (used to locate the population in the AA layout).

}  // namespace lbmg
