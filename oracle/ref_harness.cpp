// Test infrastructure: the reference CPU solver itself, driven through its own C++ API.
//
// This translation unit is compiled against the reference's unmodified headers
// (include/ of hackerbruecke/lbm, located by oracle/Makefile) plus the two inert boost stand-ins
// under oracle/stubs/. It exports one extern "C" function so that Python tests and the fixture
// generator can run a scenario exactly the way the reference driver does:
//
//   Domain ctor (domain.hpp:86-98) -> solid cells (vtk.hpp:186-195 or setBoundaryCondition)
//   -> BoundaryKeeper::get_collision + setBoundaryCondition per boundary (scenario.h:183-186,
//   domain.hpp:174-194) -> set_nonfluid_cells_nullcollide (main.cpp:40)
//   -> T x { stream(); swap(); collide(); } timed like main.cpp:47-53.
//
// Nothing here is part of the product: only tests, smoke() and bench.py's CPU arm load it.

#include <cassert>
#include <cstdint>
#include <list>
#include <memory>
#include <omp.h>

#include "model.h"
#include "parallel.h"
#include "lbmdefinitions.h"
#include "helper.h"
#include "collision.h"
#include "boundary.h"
#include "cell.h"
#include "domain.h"

namespace {

// Boundary condition codes, shared with oracle/lbm_oracle.h and include/lbm_gb300.h.
enum : int {
    kNoSlip = 1, kMovingWall = 2, kFreeSlip = 3, kOutflow = 4, kInflow = 5, kPressure = 6
};

template <typename M>
int run(int xl, int yl, int zl, double tau, int nbc, const int* bc_type, const double* bc_param,
        const int64_t* bc_box, const unsigned char* solid, int solid_mode, const double* init,
        int steps, int threads, double* out_pops, double* out_rho, double* out_u,
        double* out_seconds)
{
    using namespace lbm;
    if (threads > 0) omp_set_num_threads(threads);
    BGKCollision<M> bgk(tau);
    auto domain = std::unique_ptr<Domain<M>>(new Domain<M>(xl, yl, zl, bgk));
    const size_t Q = M::Q;

    if (solid) {
        auto& ns = BoundaryKeeper<M>::template get_collision<NoSlipBoundary<M>>(*domain);
        size_t i = 0;
        for (int z = 1; z <= zl; ++z)
            for (int y = 1; y <= yl; ++y)
                for (int x = 1; x <= xl; ++x, ++i) {
                    if (!solid[i]) continue;
                    if (solid_mode == 1)
                        domain->cell(x, y, z).set_collision_handler(&ns);   // vtk.hpp:193-195
                    else
                        domain->setBoundaryCondition(ns, x, x, y, y, z, z);
                }
    }
    for (int b = 0; b < nbc; ++b) {
        const double* p = bc_param + 4 * b;
        const int64_t* e = bc_box + 6 * b;
        const double_array<3> v = { p[0], p[1], p[2] };
        NonFluidCollision<M>* c = nullptr;
        switch (bc_type[b]) {
        case kNoSlip:
            c = &BoundaryKeeper<M>::template get_collision<NoSlipBoundary<M>>(*domain); break;
        case kMovingWall:
            c = &BoundaryKeeper<M>::template get_collision<MovingWallBoundary<M>>(*domain, v); break;
        case kFreeSlip:
            c = &BoundaryKeeper<M>::template get_collision<FreeSlipBoundary<M>>(*domain); break;
        case kOutflow:
            c = &BoundaryKeeper<M>::template get_collision<OutflowBoundary<M>>(*domain, p[3]); break;
        case kInflow:
            c = &BoundaryKeeper<M>::template get_collision<InflowBoundary<M>>(*domain, v, p[3]);
            break;
        case kPressure:
            c = &BoundaryKeeper<M>::template get_collision<PressureBoundary<M>>(*domain, p[3]);
            break;
        default:
            return -1;
        }
        domain->setBoundaryCondition(*c, e[0], e[1], e[2], e[3], e[4], e[5]);
    }
    if (init) {
        size_t i = 0;
        for (int z = 0; z < zl + 2; ++z)
            for (int y = 0; y < yl + 2; ++y)
                for (int x = 0; x < xl + 2; ++x, ++i)
                    for (size_t q = 0; q < Q; ++q) domain->cell(x, y, z)[q] = init[i * Q + q];
    }
    domain->set_nonfluid_cells_nullcollide();

    double seconds = 0.0;
    for (int t = 1; t <= steps; ++t) {
        const double start = omp_get_wtime();
        domain->stream();
        domain->swap();
        domain->collide();
        seconds += omp_get_wtime() - start;
    }
    if (out_seconds) *out_seconds = seconds;

    if (out_pops) {
        size_t i = 0;
        for (int z = 0; z < zl + 2; ++z)
            for (int y = 0; y < yl + 2; ++y)
                for (int x = 0; x < xl + 2; ++x, ++i)
                    for (size_t q = 0; q < Q; ++q) out_pops[i * Q + q] = domain->cell(x, y, z)[q];
    }
    if (out_rho || out_u) {
        // Same per-cell calls as the VTK writer (vtk.hpp:62-73): interior cells, x fastest.
        size_t i = 0;
        for (int z = 1; z <= zl; ++z)
            for (int y = 1; y <= yl; ++y)
                for (int x = 1; x <= xl; ++x, ++i) {
                    const auto& c = domain->cell(x, y, z);
                    const double rho = c.density();
                    const auto u = c.velocity(rho);
                    if (out_rho) out_rho[i] = rho;
                    if (out_u) { out_u[3 * i] = u[0]; out_u[3 * i + 1] = u[1]; out_u[3 * i + 2] = u[2]; }
                }
    }
    return 0;
}

}  // namespace

extern "C" int ref_run(int q, int xl, int yl, int zl, double tau, int nbc, const int* bc_type,
                       const double* bc_param, const int64_t* bc_box, const unsigned char* solid,
                       int solid_mode, const double* init, int steps, int threads,
                       double* out_pops, double* out_rho, double* out_u, double* out_seconds)
{
    try {
        switch (q) {
        case 15:
            return run<lbm::model::d3q15>(xl, yl, zl, tau, nbc, bc_type, bc_param, bc_box, solid,
                                          solid_mode, init, steps, threads, out_pops, out_rho,
                                          out_u, out_seconds);
        case 19:
            return run<lbm::model::d3q19>(xl, yl, zl, tau, nbc, bc_type, bc_param, bc_box, solid,
                                          solid_mode, init, steps, threads, out_pops, out_rho,
                                          out_u, out_seconds);
        case 27:
            return run<lbm::model::d3q27>(xl, yl, zl, tau, nbc, bc_type, bc_param, bc_box, solid,
                                          solid_mode, init, steps, threads, out_pops, out_rho,
                                          out_u, out_seconds);
        default:
            return -1;
        }
    } catch (...) {
        return -2;
    }
}

extern "C" double ref_cs() { return lbm::C_S; }
