// Per-(lattice, storage precision) kernel launchers, reached through a table of function
// pointers so that the host layer (capi.cu) stays free of templates and each precision lives in
// its own translation unit.
#pragma once

#include <cuda_runtime.h>

#include "domain.cuh"

namespace lbmg {

struct KernelOps {
    // all planes <- initial weights
    void (*init)(const DomainDev& d, cudaStream_t s);
    // fluid cells -> kFluidBulk / kFluidEdge
    void (*classify)(const DomainDev& d, cudaStream_t s);
    // one time step number `t` (1-based): fused kernel, then the side passes. Monitored steps
    // (mon_set 0 or 1; -1: none) add the FP64 mass and momentum the step started from into that
    // accumulator set, and with prev_out the step's first block first folds the other set (the
    // previous monitored step's) into prev_out (device, 4 doubles). With rec (device, 4
    // compute-type values per cell) each cell's pre-collision mass and momentum.
    void (*step)(const DomainDev& d, long long t, int mon_set, double* prev_out, void* rec, cudaStream_t s);
    // folds accumulator set mon_set into out (device, 4 doubles): the last monitored step of a call
    void (*monitor_fold)(const DomainDev& d, int mon_set, double* out, cudaStream_t s);
    // state after `k` steps -> AoS FP64 over all cells (device buffer)
    void (*gather)(const DomainDev& d, long long k, double* out, cudaStream_t s);
    // AoS FP64 over all cells (device buffer) -> state after `k` steps
    void (*scatter)(const DomainDev& d, long long k, const double* in, cudaStream_t s);
    // interior moments (device buffers)
    void (*moments)(const DomainDev& d, long long k, double* rho, double* u, cudaStream_t s);
    // chunked host transfers through staging buffers: rows [r0, r1) of the AoS FP64 field (reference
    // cell order) out of / into the state after `k` steps (ghost-fluid cells excluded), and the
    // moments of the interior cells [n0, n1) (interior order)
    void (*gather_range)(const DomainDev& d, long long k, size_t r0, size_t r1, double* out, cudaStream_t s);
    void (*scatter_range)(const DomainDev& d, long long k, size_t r0, size_t r1, const double* in, cudaStream_t s);
    void (*moments_range)(const DomainDev& d, long long k, size_t n0, size_t n1, double* rho, double* u,
                          cudaStream_t s);
    // the boundary slots fed by the ghost-fluid cells, from their side copy for step parity k & 1
    void (*ghost_fluid_slots)(const DomainDev& d, long long k, cudaStream_t s);
    // FP64 totals into out[4] (device), partials: scratch of 4 * reduce_blocks doubles
    void (*reduce)(const DomainDev& d, long long k, double* partials, int reduce_blocks,
                   double* out, cudaStream_t s);
    // adjoint (compute type: double for FP64 storage, float otherwise)
    size_t compute_bytes;
    // mu_T from the final step's record and the objective box
    void (*adj_terminal)(const DomainDev& d, const void* rec, void* mu_out, Box box, cudaStream_t s);
    // mu_t -> mu_{t-1} with the record of step t-1; theta gradients of step t
    void (*adj_step)(const DomainDev& d, const void* mu_in, void* mu_out, const void* rec, int bc_terms,
                     int write_mu, double* grad_inflow, double* grad_wall, cudaStream_t s);
    // LinkRecords of the kFluidWall cells with non-no-slip links (capacity 0: count only)
    void (*link_table)(const DomainDev& d, LinkRecord* ltab, int* counter, int capacity, cudaStream_t s);
    // kinetic energy of the box into out[0] (device), partials as for reduce
    void (*objective_ke)(const DomainDev& d, long long k, Box box, double* partials, int reduce_blocks,
                         double* out, cudaStream_t s);
    // the step kernel's per-segment warp mask (d.flag classified) into out, one byte per segment
    // (row_segments(d.g, row_cells))
    void (*warp_mask)(const DomainDev& d, uint8_t* out, cudaStream_t s);
    // cells per row segment of the step kernel
    int row_cells;
};

// Row segments of the step kernel: ceil(xl / row_cells) per row, rows in (y, z) order.
inline size_t row_segments(const Geom& g, int row_cells)
{
    return static_cast<size_t>((g.xl + row_cells - 1) / row_cells) * g.yl * g.zl;
}

const KernelOps* ops_fp64(int q);
const KernelOps* ops_fp32(int q);
const KernelOps* ops_fp16(int q);
const KernelOps* ops_bf16(int q);

// Blocks used by the reduction: a fixed grid, so the summation order never changes.
constexpr int kReduceBlocks = 4 * 152;

}  // namespace lbmg
