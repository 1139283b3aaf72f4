// The reference driver's time loop (src/main.cpp:34-66) written against the reference's API,
// compiled against include/lbm_gb300.hpp instead of the reference headers. Builds the
// cavity.xml face sequence through BoundaryKeeper / setBoundaryCondition (scenario.h:183-186),
// steps with stream(); swap(); collide(); and writes density and velocity of every interior cell
// (the VTK writer's loop, vtk.hpp:62-73) as raw doubles: rho[n], then u[3n].
//
//   cavity_drop_in <xl> <yl> <zl> <steps> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lbm_gb300.hpp"

using model = lbm::model::d3q19;

int main(int argc, char** argv)
{
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s xl yl zl steps out.bin\n", argv[0]);
        return 2;
    }
    const size_t xl = std::strtoul(argv[1], nullptr, 10), yl = std::strtoul(argv[2], nullptr, 10),
                 zl = std::strtoul(argv[3], nullptr, 10);
    const unsigned steps = std::strtoul(argv[4], nullptr, 10);
    try {
        auto collision = lbm::BGKCollision<model>(0.6);
        lbm::Domain<model> domain(xl, yl, zl, collision);
        using BK = lbm::BoundaryKeeper<model>;
        auto& z0 = BK::get_collision<lbm::NoSlipBoundary<model>>(domain);
        domain.setBoundaryCondition(z0, 0, xl + 1, 0, yl + 1, 0, 0);
        auto& lid = BK::get_collision<lbm::MovingWallBoundary<model>>(domain, lbm::double_array<3>{0.05, 0, 0});
        domain.setBoundaryCondition(lid, 0, xl + 1, 0, yl + 1, zl + 1, zl + 1);
        auto& x0 = BK::get_collision<lbm::NoSlipBoundary<model>>(domain);
        domain.setBoundaryCondition(x0, 0, 0, 0, yl + 1, 0, zl + 1);
        auto& xm = BK::get_collision<lbm::NoSlipBoundary<model>>(domain);
        domain.setBoundaryCondition(xm, xl + 1, xl + 1, 0, yl + 1, 0, zl + 1);
        auto& y0 = BK::get_collision<lbm::NoSlipBoundary<model>>(domain);
        domain.setBoundaryCondition(y0, 0, xl + 1, 0, 0, 0, zl + 1);
        auto& ym = BK::get_collision<lbm::NoSlipBoundary<model>>(domain);
        domain.setBoundaryCondition(ym, 0, xl + 1, yl + 1, yl + 1, 0, zl + 1);
        domain.set_nonfluid_cells_nullcollide();
        for (unsigned t = 1; t <= steps; ++t) {
            domain.stream();
            domain.swap();
            domain.collide();
        }
        const auto& cdom = domain;
        std::vector<double> rho, u;
        for (size_t z = 1; z < zl + 1; ++z)
            for (size_t y = 1; y < yl + 1; ++y)
                for (size_t x = 1; x < xl + 1; ++x) {
                    const auto& c = cdom.cell(x, y, z);
                    const double r = c.density();
                    const auto v = c.velocity(r);
                    rho.push_back(r);
                    u.insert(u.end(), v.begin(), v.end());
                }
        FILE* f = std::fopen(argv[5], "wb");
        if (!f) return 3;
        std::fwrite(rho.data(), sizeof(double), rho.size(), f);
        std::fwrite(u.data(), sizeof(double), u.size(), f);
        std::fclose(f);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "An error occured: %s\n", ex.what());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
