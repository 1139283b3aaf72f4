/*
 * lbm_gb300.h -- C ABI of the GB300 lattice Boltzmann step library (liblbm_gb300.so).
 *
 * This is the drop-in boundary for the time loop of hackerbruecke/lbm. The reference exposes a
 * header-only C++ template API (lbm::Domain, lbm::BGKCollision, the boundary handlers,
 * lbm::BoundaryKeeper); every entry point below names the reference call it replaces. Plain
 * pointers and sizes only: no C++ or torch types cross this boundary, and no exception escapes it.
 *
 * Conventions
 *   - Every function returns LBM_OK (0) or an LBM_ERR_* code; lbm_last_error() gives the text.
 *     The reference reports the same conditions with assert() and std::logic_error
 *     (configuration.h:123-128, domain.hpp:180-181, scenario.h:21-26).
 *   - Cell coordinates follow the reference: interior cells are 1..xl (resp. yl, zl), the ghost
 *     layer is 0 and xl+1; host arrays over "all cells" use the reference's cell order
 *     x + (xl+2)*(y + (yl+2)*z) (domain.hpp:60-64); arrays over "interior cells" use
 *     (x-1) + xl*((y-1) + yl*(z-1)), the VTK writer's order (vtk.hpp:62-73).
 *   - Populations are exchanged as FP64 whatever the storage precision.
 *   - A handle owns its device memory and one CUDA stream (plus a copy stream for the chunked
 *     host transfers) on the device that was current at lbm_create; all work is ordered on that
 *     stream. Every call makes the handle's device current while it runs and restores the
 *     caller's current device before returning. lbm_step() is asynchronous; the read-back calls
 *     synchronise. One handle per host thread.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define LBM_OK            0
#define LBM_ERR_ARG       1  /* invalid argument (reference: assert / std::logic_error)       */
#define LBM_ERR_OOM       2  /* device or host allocation failed                               */
#define LBM_ERR_CUDA      3  /* a CUDA runtime call failed                                     */
#define LBM_ERR_DIVERGED  4  /* non-finite mass or momentum found by lbm_reduce_mass_momentum */
#define LBM_ERR_STATE     5  /* call not valid in the current state                            */

/* Boundary conditions: the reference's NonFluidCollision subclasses (boundary.h:10-70). */
#define LBM_NOSLIP      1  /* NoSlipBoundary      boundary.hpp:14-31                  */
#define LBM_MOVINGWALL  2  /* MovingWallBoundary  boundary.hpp:43-68   (vx, vy, vz)   */
#define LBM_FREESLIP    3  /* FreeSlipBoundary    boundary.hpp:79-115                 */
#define LBM_OUTFLOW     4  /* OutflowBoundary     boundary.hpp:128-150 (rho-ref)      */
#define LBM_INFLOW      5  /* InflowBoundary      boundary.hpp:164-181 (vx,vy,vz,rho) */
#define LBM_PRESSURE    6  /* PressureBoundary    boundary.hpp:194-214 (rho-in)       */

/* Population storage precision. Arithmetic is FP64 for LBM_FP64 and FP32 otherwise; the
 * FP32/FP16/BF16 stores hold f_q - w_q (shifted by the lattice weight). */
#define LBM_FP64  0
#define LBM_FP32  1
#define LBM_FP16  2
#define LBM_BF16  3

typedef struct lbm_domain lbm_domain;

/* Domain<M>(xl, yl, zl, BGKCollision<M>(tau)) -- domain.hpp:86-98, collision.hpp:54-58.
 * q selects the lattice model (15, 19 or 27: model.h:13-139); tau must lie in (0.5, 2.0)
 * (configuration.h:124). All populations start at the weights (cell.hpp:8-15); ghost cells
 * start as fluid cells, as in the reference. */
int lbm_create(lbm_domain** out, int q, int64_t xl, int64_t yl, int64_t zl, double tau,
               int precision);

/* Releases the handle and its device memory. */
void lbm_destroy(lbm_domain* d);

/* BoundaryKeeper<M>::get_collision<BC>(domain, args...) -- boundary.h:85-91. params holds
 * {vx, vy, vz, rho}: the wall/inflow velocity and rho-ref (inflow, outflow) or rho-in
 * (pressure); unused entries are ignored. *handler receives the handler id (>= 1). At most
 * 250 handlers per domain. */
int lbm_add_boundary(lbm_domain* d, int type, const double params[4], int* handler);

/* Domain::setBoundaryCondition(handler, x0, xE, y0, yE, z0, zE) -- domain.hpp:174-194.
 * box = {x0, xE, y0, yE, z0, zE}, inclusive, may include ghost cells; later calls overwrite
 * earlier ones cell by cell (edges and corners: last writer wins). */
int lbm_set_boundary_box(lbm_domain* d, int handler, const int64_t box[6]);

/* Solid interior cells bound to a fresh no-slip handler, as io::read_vtk_point_file does for
 * mask value 0 (vtk.hpp:186-195). mask covers the interior cells (interior order), nonzero =
 * solid. Unlike vtk.hpp:195, which installs the handler in collide_field only, the cells are
 * solid in both lattice fields. *handler (may be NULL) receives the handler id. */
int lbm_set_solid_mask(lbm_domain* d, const uint8_t* mask, int* handler);

/* Extension (no reference counterpart): periodic axes. Pulls and boundary-neighbour lookups
 * wrap around 1..l on each axis whose flag is nonzero; that axis's ghost cells are unused. */
int lbm_set_periodic(lbm_domain* d, int px, int py, int pz);

/* Extension (no reference counterpart): per-cell inflow velocity for an LBM_INFLOW handler.
 * u_cells holds 3 doubles per cell over all cells (reference cell order); only cells that carry
 * this handler are read. */
int lbm_set_inflow_profile(lbm_domain* d, int handler, const double* u_cells);

/* Domain::set_nonfluid_cells_nullcollide() -- domain.hpp:100-113. The reference uses it to skip
 * solid cells without fluid neighbours; the result is unchanged by it, and this library skips
 * those cells anyway, so the call only records that it was made. */
int lbm_set_nonfluid_cells_nullcollide(lbm_domain* d);

/* Writes the current populations (the reference's collide_field, Domain::cell(x,y,z)[q],
 * domain.hpp:73-83) from a host array of Q doubles per cell over all cells. The array is moved
 * in chunks through two staging buffers of the handle (at most 32 MiB each, allocated by the
 * first transfer call and kept until lbm_destroy), each chunk's copy overlapping the previous
 * chunk's conversion on the device; page-locked host memory makes the copies asynchronous.
 * Synchronises. */
int lbm_set_populations(lbm_domain* d, const double* f);

/* Reads the current populations (collide_field) into a host array of Q doubles per cell over
 * all cells. Fluid cells hold their post-collision values; boundary cells hold what their
 * handler wrote in the last collide (boundary.hpp) in every direction that faces an interior
 * fluid cell, and the initial weight w_q in the other directions. Chunked through the staging
 * buffers as lbm_set_populations. Synchronises. */
int lbm_get_populations(lbm_domain* d, double* f);

/* nsteps x { Domain::stream(); Domain::swap(); Domain::collide(); } -- domain.hpp:115-172,
 * main.cpp:48-53. One fused kernel per step (pull-stream, BGK collide, boundary handlers) on the
 * handle's stream. Asynchronous: returns after the launches. */
int lbm_step(lbm_domain* d, int64_t nsteps);

/* Extension: lbm_step with a conservation monitor. Each step also reduces, inside the step kernel,
 * the FP64 totals of the populations it pulled (the mass and momentum it started from: sum rho,
 * sum j_x, sum j_y, sum j_z over interior fluid cells: each block adds its partial sums to FP64
 * accumulators, which the next step's first block, or a one-block kernel after the call's last
 * step, adds up) into a device ring of 1024 slots, which is copied asynchronously to
 * totals[4*k .. 4*k+3] (the k-th step of the call) once per 1024 steps and after the last step.
 * totals must hold 4*nsteps doubles and stay valid until the next synchronising call; page-locked
 * host memory keeps the copies asynchronous. The totals are summed with atomics, so their last
 * bits may differ between runs.
 * FP16 / BF16 / FP32 storage: each warp first sums its 32 cells' rho - 1 and j in FP32 (absolute
 * error of order 1e-8 per warp), and the warp sums are accumulated in FP64. FP64 storage sums in
 * FP64 throughout. */
int lbm_step_monitored(lbm_domain* d, int64_t nsteps, double* totals);

/* Density and velocity of every interior cell (Cell::density / Cell::velocity on
 * collide_field, vtk.hpp:62-73), computed on the device in FP64. rho: one double per interior
 * cell; u: three (may be NULL). Chunked through the staging buffers as lbm_set_populations (the
 * first transfer call of a handle allocates them). Synchronises. */
int lbm_moments(lbm_domain* d, double* rho, double* u);

/* No counterpart in the reference: lbm_moments for callers that must not allocate device memory.
 * Same results as lbm_moments (the same arithmetic), but the device buffer that holds the moments
 * on their way to the host is a static array inside the library (8 MiB, at most 262144 interior
 * cells; larger domains are rejected with LBM_ERR_ARG) instead of the staging buffers that
 * lbm_moments allocates on a handle's first transfer. For callers whose device memory is owned by
 * their own pool allocator: a cudaMalloc would fail once the pool holds all free memory, or would
 * make the pool give memory back, and a cudaMalloc / cudaFree pair synchronises the whole device.
 *   - The first call on a device looks up the array's device address (cudaGetSymbolAddress);
 *     make that first call before any stream capture.
 *   - All calls in the process share the array: calls whose work overlaps on the GPU (two handles
 *     on different streams) race. Each call writes every element it reads back, so nothing
 *     carries over from the previous call.
 *   - Returns LBM_ERR_STATE when the geometry changed since the last step (applying the change
 *     may allocate); any call that steps or reads the state applies it first.
 * The array stays allocated in every GPU that loads the library until the process exits. */
int lbm_moments_noalloc(lbm_domain* d, double* rho, double* u);

/* Extension: FP64 totals over interior fluid cells of the post-collision populations:
 * out = {sum rho, sum j_x, sum j_y, sum j_z}. Returns LBM_ERR_DIVERGED (after filling out) when
 * any total is not finite. Synchronises. */
int lbm_reduce_mass_momentum(lbm_domain* d, double out[4]);

/* Extension (no reference counterpart): gradients by a hand-written discrete adjoint of the step.
 * Forward: nsteps steps from the current state, keeping a copy of the state every ckpt_every
 * steps (device memory: ceil(nsteps / ckpt_every) copies of the population store). ckpt_every = 1
 * keeps no state copies: every step records each cell's mass and momentum instead (4 values per
 * cell and step in the compute type, nsteps records; LBM_ERR_OOM if they do not fit), which is
 * all the backward needs, so it then recomputes nothing. Not available with free-slip cells or
 * ghost cells without a handler (LBM_ERR_STATE). */
int lbm_adjoint_forward(lbm_domain* d, int64_t nsteps, int64_t ckpt_every);

/* J = sum over the interior fluid cells of box = {x0, xE, y0, yE, z0, zE} (inclusive, interior
 * coordinates) of rho |u|^2 / 2, from the current post-collision populations, FP64. */
int lbm_adjoint_objective_ke(lbm_domain* d, const int64_t box[6], double* J);

/* dJ/dtheta of the objective of box at the end of the last lbm_adjoint_forward, times dJ (the
 * upstream gradient when wrapped in an autodiff framework), with the state the run started from
 * held fixed. That state includes the boundary values its first step pulls (computed by the step
 * before it, as in the reference), so theta acts through the run's steps 2 .. n. Recomputes each
 * checkpoint segment while recording per-cell mass and momentum, then runs the adjoint steps
 * backwards through it.
 * grad_inflow (may be NULL): 3 doubles per cell over all cells (reference cell order), the
 * gradient with respect to the inflow velocity of each inflow cell (the per-cell profile or the
 * handler's uniform velocity at that cell); grad_wall (may be NULL): 3 doubles per handler id
 * (1-based id h at index 3*(h-1)), the gradient with respect to each moving wall's velocity. The
 * state is left as lbm_adjoint_forward left it, so the call may be repeated (another box or dJ).
 * Device memory (allocated by the first call and kept with the handle for the next ones, until a
 * geometry change, a run with another checkpoint interval, or lbm_destroy): two adjoint population
 * stores (Q values per cell in the compute type: FP32, or FP64 for FP64 storage), 2 * ckpt_every * 4
 * recorded values per cell (the recompute of one checkpoint segment overlaps the adjoint steps of
 * the next), one copy of the population store and 3 doubles per cell (after a
 * ckpt_every = 1 forward: the adjoint stores and the gradients only, beside its records). The
 * gradients are scaled by dJ on the device and copied into the caller's arrays. Synchronises. */
int lbm_adjoint_backward(lbm_domain* d, const int64_t box[6], double dJ, double* grad_inflow,
                         double* grad_wall);

/* Blocks until all work queued on the handle's stream has finished. */
int lbm_sync(lbm_domain* d);

/* The handle's cudaStream_t, as a void*. */
int lbm_get_stream(lbm_domain* d, void** stream);

/* Number of completed time steps since creation. */
int64_t lbm_steps_done(const lbm_domain* d);

/* Device bytes held by the handle, the algorithmic HBM bytes of one step (2*Q*s per interior
 * fluid cell: one read and one write of every population), the number of interior fluid cells
 * and the number of kernel launches one step makes. Any pointer may be NULL. */
int lbm_memory_info(const lbm_domain* d, uint64_t* device_bytes, uint64_t* step_bytes,
                    uint64_t* fluid_cells, uint64_t* launches_per_step);

/* Text of the last error on this handle (or of the last failed lbm_create when d is NULL). */
const char* lbm_last_error(const lbm_domain* d);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
