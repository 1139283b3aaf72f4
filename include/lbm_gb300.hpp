// lbm_gb300.hpp -- drop-in C++ interface of the GB300 lattice Boltzmann library.
//
// The same names, signatures and behaviour as the reference's header-only API (hackerbruecke/lbm
// include/model.h, lbmdefinitions.h, cell.h, collision.h, boundary.h, domain.h), implemented on
// the C ABI of include/lbm_gb300.h. A program written against the reference, e.g. its driver
// (src/main.cpp:30-73), compiles against this header instead and runs its time loop on the GPU:
//
//   lbm::BGKCollision<model> collision(tau);
//   lbm::Domain<model> domain(xl, yl, zl, collision);
//   auto& lid = lbm::BoundaryKeeper<model>::get_collision<lbm::MovingWallBoundary<model>>(domain, v);
//   domain.setBoundaryCondition(lid, 0, xl + 1, 0, yl + 1, zl + 1, zl + 1);
//   domain.set_nonfluid_cells_nullcollide();
//   for (...) { domain.stream(); domain.swap(); domain.collide(); }
//
// stream() and swap() record the call; collide() launches the fused step (one kernel), so the
// three must come in the reference's order (anything else throws std::logic_error). Cell access
// (domain.cell(x, y, z)[q], density(), velocity()) works on a host copy of collide_field that is
// read from the device on first use after a step and written back before the next step when it
// was accessed through a non-const Domain. Errors throw std::logic_error with the library's text,
// as the reference's parser does (scenario.h:21-26).
#pragma once

#include <array>
#include <cstdint>
#include <list>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lbm_gb300.h"

namespace lbm {

// lbmdefinitions.h:9-47
template <size_t SIZE>
using double_array = std::array<double, SIZE>;
template <size_t SIZE>
using int_array = std::array<int, SIZE>;
template <size_t SIZE>
using uint_array = std::array<std::uint64_t, SIZE>;
template <size_t SIZE>
using lattice_weights = std::array<double, SIZE>;

// 0.57735026919l converted to double, as lbmdefinitions.h:47 defines it
static constexpr double C_S = 0x1.279a745904047p-1;

namespace model {

// model.h:13-50
struct d3q15 {
    static constexpr size_t D = 3;
    static constexpr size_t Q = 15;
    static constexpr const char* const name = "D3Q15";
    static constexpr double velocities[Q][D]{
        {-1, -1, -1}, {1, -1, -1}, {0, 0, -1}, {-1, 1, -1}, {1, 1, -1}, {0, -1, 0}, {-1, 0, 0}, {0, 0, 0},
        {1, 0, 0},    {0, 1, 0},   {-1, -1, 1}, {1, -1, 1}, {0, 0, 1},  {-1, 1, 1}, {1, 1, 1}};
    static constexpr lattice_weights<Q> weights{{1.0 / 72, 1.0 / 72, 8.0 / 72, 1.0 / 72, 1.0 / 72, 8.0 / 72,
                                                 8.0 / 72, 16.0 / 72, 8.0 / 72, 8.0 / 72, 1.0 / 72, 1.0 / 72,
                                                 8.0 / 72, 1.0 / 72, 1.0 / 72}};
    static int inv(int q) { return Q - 1 - q; }
    static size_t velocity_index(int u, int v, int w) { return 5 * w + 2 * v + u + 7 - (w + 2) % 2 * (u + v) / 2; }
};

// model.h:53-91
struct d3q19 {
    static constexpr size_t D = 3;
    static constexpr size_t Q = 19;
    static constexpr const char* const name = "D3Q19";
    static constexpr double velocities[Q][D]{
        {0, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {0, 1, -1}, {-1, -1, 0}, {0, -1, 0},
        {1, -1, 0},  {-1, 0, 0},  {0, 0, 0},  {1, 0, 0},  {-1, 1, 0}, {0, 1, 0},   {1, 1, 0},
        {0, -1, 1},  {-1, 0, 1},  {0, 0, 1},  {1, 0, 1},  {0, 1, 1}};
    static constexpr lattice_weights<Q> weights{{1.0 / 36, 1.0 / 36, 2.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                                                 2.0 / 36, 1.0 / 36, 2.0 / 36, 12.0 / 36, 2.0 / 36, 1.0 / 36,
                                                 2.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 2.0 / 36, 1.0 / 36,
                                                 1.0 / 36}};
    static int inv(int q) { return Q - 1 - q; }
    static size_t velocity_index(int u, int v, int w)
    {
        return w == 0 ? (6 + (v + 1) * 3 + u) : ((w + 1) * 7 + (v + 1) * 2 + u);
    }
};

// model.h:96-139
struct d3q27 {
    static constexpr size_t D = 3;
    static constexpr size_t Q = 27;
    static constexpr const char* const name = "D3Q27";
    static constexpr double velocities[Q][D]{
        {-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {-1, 1, -1},
        {0, 1, -1},   {1, 1, -1},  {-1, -1, 0}, {0, -1, 0},  {1, -1, 0}, {-1, 0, 0}, {0, 0, 0},
        {1, 0, 0},    {-1, 1, 0},  {0, 1, 0},   {1, 1, 0},   {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
        {-1, 0, 1},   {0, 0, 1},   {1, 0, 1},   {-1, 1, 1},  {0, 1, 1},  {1, 1, 1}};
    static constexpr lattice_weights<Q> weights{
        {1.0 / 216,  4.0 / 216,  1.0 / 216, 4.0 / 216,  16.0 / 216, 4.0 / 216, 1.0 / 216,
         4.0 / 216,  1.0 / 216,  4.0 / 216, 16.0 / 216, 4.0 / 216,  16.0 / 216, 64.0 / 216,
         16.0 / 216, 4.0 / 216,  16.0 / 216, 4.0 / 216, 1.0 / 216,  4.0 / 216, 1.0 / 216,
         4.0 / 216,  16.0 / 216, 4.0 / 216, 1.0 / 216,  4.0 / 216,  1.0 / 216}};
    static int inv(int q) { return Q - 1 - q; }
    static size_t velocity_index(int u, int v, int w) { return 9 * w + 3 * v + u + 13; }
};

}  // namespace model

namespace detail {
inline void check(int rc, const lbm_domain* d)
{
    if (rc != LBM_OK) throw std::logic_error(std::string("lbm_gb300: ") + lbm_last_error(d));
}
}  // namespace detail

template <typename M> class Cell;
template <typename M> class Domain;

// collision.h:18-31: moments and equilibrium of a cell (host side, the reference's formulas)
template <typename M>
class Collision {
public:
    double compute_density(const Cell<M>& cell) const
    {
        double density = 0;
        for (size_t q = 0; q < M::Q; ++q) density += cell[q];
        return density;
    }
    double_array<M::D> compute_velocity(const Cell<M>& cell, double density) const
    {
        double_array<M::D> v = {0.0, 0.0, 0.0};
        for (size_t d = 0; d < M::D; ++d)
            for (size_t q = 0; q < M::Q; ++q) v[d] += cell[q] * M::velocities[q][d];
        v[0] /= density;
        v[1] /= density;
        v[2] /= density;
        return v;
    }
    double_array<M::Q> compute_feq(double density, const double_array<M::D>& u) const
    {
        double_array<M::Q> feq;
        for (size_t q = 0; q < M::Q; ++q) {
            double cu = 0.0, uu = 0.0;
            for (size_t d = 0; d < M::D; ++d) {
                cu += M::velocities[q][d] * u[d];
                uu += u[d] * u[d];
            }
            feq[q] = M::weights[q] * density *
                     (1 + cu / (C_S * C_S) + cu * cu / (2 * C_S * C_S * C_S * C_S) - uu / (2 * C_S * C_S));
        }
        return feq;
    }
    virtual bool is_fluid() const = 0;
    virtual ~Collision() {}
};

template <typename M>
class FluidCollision : public Collision<M> {
public:
    bool is_fluid() const override final { return true; }
    virtual double relaxation_time() const = 0;
};

// collision.h:63-71
template <typename M>
class BGKCollision : public FluidCollision<M> {
    double tau{0};

public:
    explicit BGKCollision(double tau) : tau{tau} {}
    double relaxation_time() const override { return tau; }
};

// collision.h:36-54: a handler bound to one domain; here one handler id of that domain
template <typename M>
class NonFluidCollision : public Collision<M> {
protected:
    Domain<M>& domain;
    int handler_{0};
    NonFluidCollision(Domain<M>& domain, int type, double vx, double vy, double vz, double rho) : domain(domain)
    {
        const double p[4] = {vx, vy, vz, rho};
        detail::check(lbm_add_boundary(domain.native(), type, p, &handler_), domain.native());
    }

public:
    bool is_fluid() const override final { return false; }
    int handler() const { return handler_; }
    Domain<M>& owner() const { return domain; }
};

// boundary.h:10-70
template <typename M>
class NoSlipBoundary : public NonFluidCollision<M> {
public:
    explicit NoSlipBoundary(Domain<M>& d) : NonFluidCollision<M>(d, LBM_NOSLIP, 0, 0, 0, 1.0) {}
};
template <typename M>
class MovingWallBoundary : public NonFluidCollision<M> {
public:
    MovingWallBoundary(Domain<M>& d, const double_array<M::D>& v)
        : NonFluidCollision<M>(d, LBM_MOVINGWALL, v[0], v[1], v[2], 1.0) {}
};
template <typename M>
class FreeSlipBoundary : public NonFluidCollision<M> {
public:
    explicit FreeSlipBoundary(Domain<M>& d) : NonFluidCollision<M>(d, LBM_FREESLIP, 0, 0, 0, 1.0) {}
};
template <typename M>
class OutflowBoundary : public NonFluidCollision<M> {
public:
    OutflowBoundary(Domain<M>& d, double reference_density = 1.0)
        : NonFluidCollision<M>(d, LBM_OUTFLOW, 0, 0, 0, reference_density) {}
};
template <typename M>
class InflowBoundary : public NonFluidCollision<M> {
public:
    InflowBoundary(Domain<M>& d, const double_array<M::D>& v, double reference_density = 1.0)
        : NonFluidCollision<M>(d, LBM_INFLOW, v[0], v[1], v[2], reference_density) {}
};
template <typename M>
class PressureBoundary : public NonFluidCollision<M> {
public:
    PressureBoundary(Domain<M>& d, double input_density)
        : NonFluidCollision<M>(d, LBM_PRESSURE, 0, 0, 0, input_density) {}
};

// boundary.h:72-91: handlers live for the rest of the program
template <typename M>
class BoundaryKeeper {
    static std::list<std::unique_ptr<NonFluidCollision<M>>>& store()
    {
        static std::list<std::unique_ptr<NonFluidCollision<M>>> s;
        return s;
    }

public:
    template <typename BC, typename... Args>
    static NonFluidCollision<M>& get_collision(Args&&... args)
    {
        store().push_back(std::unique_ptr<NonFluidCollision<M>>(new BC(std::forward<Args>(args)...)));
        return *store().back();
    }
};

// cell.h:12-69: populations of one cell of the host copy of collide_field
template <typename M>
class Cell {
    double_array<M::Q> pdf;
    const Collision<M>* collision;

public:
    explicit Cell(const Collision<M>* c = nullptr) : collision{c} { pdf = M::weights; }
    double& operator[](size_t q) { return pdf[q]; }
    const double& operator[](size_t q) const { return pdf[q]; }
    bool is_fluid() const { return collision == nullptr || collision->is_fluid(); }
    double density() const
    {
        double density = 0;
        for (size_t q = 0; q < M::Q; ++q) density += pdf[q];
        return density;
    }
    double_array<M::D> velocity(double density) const
    {
        double_array<M::D> v = {0.0, 0.0, 0.0};
        for (size_t d = 0; d < M::D; ++d)
            for (size_t q = 0; q < M::Q; ++q) v[d] += pdf[q] * M::velocities[q][d];
        v[0] /= density;
        v[1] /= density;
        v[2] /= density;
        return v;
    }
    void set_collision_handler(const Collision<M>* c) { collision = c; }
    const Collision<M>* get_collision_handler() const { return collision; }
};

// domain.h:10-56
template <typename M>
class Domain {
    lbm_domain* h{nullptr};
    const FluidCollision<M>* collision;
    const size_t xl{0}, yl{0}, zl{0};
    double xo, yo, zo, xs, ys, zs;
    int phase{0};  // 0 idle, 1 after stream(), 2 after swap()
    mutable std::vector<Cell<M>> mirror;
    mutable bool mirror_valid{false};
    mutable bool mirror_dirty{false};

    void pull_mirror() const
    {
        if (mirror_valid) return;
        const size_t n = (xl + 2) * (yl + 2) * (zl + 2);
        std::vector<double> f(n * M::Q);
        detail::check(lbm_get_populations(h, f.data()), h);
        mirror.assign(n, Cell<M>(collision));
        for (size_t i = 0; i < n; ++i)
            for (size_t q = 0; q < M::Q; ++q) mirror[i][q] = f[i * M::Q + q];
        mirror_valid = true;
    }
    void push_mirror() const
    {
        if (!mirror_dirty) return;
        const size_t n = mirror.size();
        std::vector<double> f(n * M::Q);
        for (size_t i = 0; i < n; ++i)
            for (size_t q = 0; q < M::Q; ++q) f[i * M::Q + q] = mirror[i][q];
        detail::check(lbm_set_populations(h, f.data()), h);
        mirror_dirty = false;
    }

public:
    Domain(size_t xl, size_t yl, size_t zl, FluidCollision<M>& c, double xorigin = 0, double yorigin = 0,
           double zorigin = 0, double xspacing = 1, double yspacing = 1, double zspacing = 1,
           int precision = LBM_FP64)
        : collision{&c}, xl{xl}, yl{yl}, zl{zl}, xo{xorigin}, yo{yorigin}, zo{zorigin}, xs{xspacing},
          ys{yspacing}, zs{zspacing}
    {
        detail::check(lbm_create(&h, static_cast<int>(M::Q), static_cast<int64_t>(xl), static_cast<int64_t>(yl),
                                 static_cast<int64_t>(zl), c.relaxation_time(), precision),
                      nullptr);
    }
    ~Domain() { lbm_destroy(h); }
    Domain(const Domain&) = delete;
    Domain& operator=(const Domain&) = delete;

    lbm_domain* native() const { return h; }

    // Extension: solid cells (mask[z][y][x] of the interior, x fastest, nonzero = solid) bound to
    // a new no-slip handler, as io::read_vtk_point_file does (vtk.hpp:135-150).
    void set_solid_mask(const std::vector<std::uint8_t>& mask)
    {
        if (mask.size() != xl * yl * zl) throw std::logic_error("lbm_gb300: mask size must be xl*yl*zl");
        push_mirror();
        int handler = 0;
        detail::check(lbm_set_solid_mask(h, mask.data(), &handler), h);
        mirror_valid = false;
    }
    // Extension: density and velocity of the interior cells (x fastest), computed on the device.
    void moments(std::vector<double>& rho, std::vector<double>& u) const
    {
        push_mirror();
        rho.resize(xl * yl * zl);
        u.resize(3 * xl * yl * zl);
        detail::check(lbm_moments(h, rho.data(), u.data()), h);
    }

    size_t xlength() const { return xl; }
    size_t ylength() const { return yl; }
    size_t zlength() const { return zl; }
    double xorigin() const { return xo; }
    double yorigin() const { return yo; }
    double zorigin() const { return zo; }
    double xspacing() const { return xs; }
    double yspacing() const { return ys; }
    double zspacing() const { return zs; }

    // domain.hpp:60-70
    int idx(int x, int y, int z) const { return x + (xl + 2) * y + (xl + 2) * (yl + 2) * z; }
    bool in_bounds(int x, int y, int z) const
    {
        return x > 0 && x < (int)xl + 1 && y > 0 && y < (int)yl + 1 && z > 0 && z < (int)zl + 1;
    }
    const Cell<M>& cell(int x, int y, int z) const
    {
        pull_mirror();
        return mirror[idx(x, y, z)];
    }
    Cell<M>& cell(int x, int y, int z)
    {
        pull_mirror();
        mirror_dirty = true;
        return mirror[idx(x, y, z)];
    }

    void set_nonfluid_cells_nullcollide() { detail::check(lbm_set_nonfluid_cells_nullcollide(h), h); }
    void setBoundaryCondition(NonFluidCollision<M>& condition, size_t x0, size_t xE, size_t y0, size_t yE,
                              size_t z0, size_t zE)
    {
        if (&condition.owner() != this) throw std::logic_error("lbm_gb300: handler belongs to another domain");
        push_mirror();
        const int64_t box[6] = {(int64_t)x0, (int64_t)xE, (int64_t)y0, (int64_t)yE, (int64_t)z0, (int64_t)zE};
        detail::check(lbm_set_boundary_box(h, condition.handler(), box), h);
        mirror_valid = false;
    }

    // domain.hpp:115-172
    void stream()
    {
        if (phase != 0) throw std::logic_error("lbm_gb300: stream() called twice without collide()");
        phase = 1;
    }
    void swap()
    {
        if (phase != 1) throw std::logic_error("lbm_gb300: swap() must follow stream()");
        phase = 2;
    }
    void collide()
    {
        if (phase != 2) throw std::logic_error("lbm_gb300: collide() must follow stream() and swap()");
        phase = 0;
        push_mirror();
        detail::check(lbm_step(h, 1), h);
        mirror_valid = false;
    }
};

}  // namespace lbm
