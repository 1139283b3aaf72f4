/*
 * lbm_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference CPU solver's hot path (hackerbruecke/lbm,
 * include/domain.hpp, collision.hpp, boundary.hpp, model.h). It is the checker the parity tests
 * compare the CUDA path against, and the CPU arm that bench.py times on the GPU host (where the
 * reference's own headers are absent). It is never linked into, called by, or a fallback for the
 * product library.
 *
 * Parity pin: tests/test_oracle_pin.py checks this port bit-for-bit against the reference's own
 * headers compiled by oracle/Makefile (oracle/_ref/libref_lbm.so, FP contraction off), and the
 * committed fixtures under tests/golden/ were produced by that reference build.
 *
 * Layout mirrors the reference: two AoS fields of (xl+2)(yl+2)(zl+2) cells with a ghost layer,
 * cell index x + (xl+2)*(y + (yl+2)*z) (domain.hpp:60-64), Q doubles per cell.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary condition codes (same numbering as include/lbm_gb300.h). */
#define ORC_NOSLIP     1
#define ORC_MOVINGWALL 2
#define ORC_FREESLIP   3
#define ORC_OUTFLOW    4
#define ORC_INFLOW     5
#define ORC_PRESSURE   6

typedef struct orc_domain orc_domain;

/* Domain<M>(xl, yl, zl, BGKCollision(tau)) -- domain.hpp:86-98; populations start at w_q. */
orc_domain* orc_create(int q, int xl, int yl, int zl, double tau);
void orc_destroy(orc_domain* d);

/* BoundaryKeeper::get_collision (boundary.h:85-91). params = {vx, vy, vz, rho}; rho is rho-ref
 * for inflow/outflow and rho-in for pressure. Returns the handler id (>= 1) or < 0 on error. */
int orc_add_boundary(orc_domain* d, int type, const double params[4]);

/* Domain::setBoundaryCondition(handler, x0, xE, y0, yE, z0, zE), inclusive box, both fields,
 * last writer wins (domain.hpp:174-194). */
int orc_set_boundary_box(orc_domain* d, int handler, const int64_t box[6]);

/* Solid interior cells (mask over xl*yl*zl, x fastest, nonzero = solid) bound to a no-slip
 * handler. mode 0: both fields (setBoundaryCondition per cell); mode 1: collide_field only,
 * as the reference's VTK mask reader does (vtk.hpp:186-195). */
int orc_set_solid(orc_domain* d, const unsigned char* mask, int mode);

/* Extension (no reference counterpart): periodic axes; pulls and handler neighbours wrap. */
int orc_set_periodic(orc_domain* d, int px, int py, int pz);

/* Extension (no reference counterpart): per-cell inflow velocity for an inflow handler,
 * an array of 3 doubles per cell over the whole padded domain. */
int orc_set_inflow_profile(orc_domain* d, int handler, const double* u_cells);

/* Read / write collide_field populations, AoS over all (xl+2)(yl+2)(zl+2) cells. */
int orc_set_populations(orc_domain* d, const double* f);
int orc_get_populations(const orc_domain* d, double* f);

/* nsteps x { stream(); swap(); collide(); } (main.cpp:48-53) with OpenMP threads (0 = keep);
 * *seconds receives the time spent in those calls, as main.cpp:49-53 measures it. */
int orc_step(orc_domain* d, int nsteps, int threads, double* seconds);

/* Density and velocity of interior cells from collide_field (vtk.hpp:62-73). */
int orc_moments(const orc_domain* d, double* rho, double* u);

/* The reference's truncated lattice speed of sound (lbmdefinitions.h:47). */
double orc_cs(void);

#ifdef __cplusplus
}
#endif

#endif
