"""Python mirror of the reference's model / domain / collision / boundary API over the C ABI.

Names, argument meaning and error behaviour follow the reference (include/domain.h,
collision.h, boundary.h of hackerbruecke/lbm):

    collision = BGKCollision(tau)
    domain = Domain(xl, yl, zl, collision, model=d3q19)
    wall = BoundaryKeeper.get_collision(NoSlipBoundary, domain)
    domain.setBoundaryCondition(wall, 0, xl + 1, 0, yl + 1, 0, 0)
    domain.set_nonfluid_cells_nullcollide()
    for t in range(T):
        domain.stream(); domain.swap(); domain.collide()

Every call goes to liblbm_gb300.so; the three time-loop calls together launch one fused step
kernel (the launch happens in collide(), after stream() and swap() were called in that order).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from . import model as _model
from .capi import LbmError, check


class Collision:
    """Base of the collision operators (collision.h:18-31)."""


class FluidCollision(Collision):
    def is_fluid(self) -> bool:
        return True


class BGKCollision(FluidCollision):
    """BGKCollision<M>(tau) (collision.h:63-71): relaxation f -= (f - feq)/tau."""

    def __init__(self, tau: float):
        self.tau = float(tau)


class NonFluidCollision(Collision):
    """Base of the boundary handlers (collision.h:36-54). Each instance is one handler id of
    its domain; setBoundaryCondition binds cells to it."""

    kind = 0

    def __init__(self, domain: "Domain", v=(0.0, 0.0, 0.0), rho: float = 1.0):
        self.domain = domain
        self.v = tuple(float(a) for a in v)
        self.rho = float(rho)
        self.handler = domain._add_handler(self.kind, self.v, self.rho)

    def is_fluid(self) -> bool:
        return False


class NoSlipBoundary(NonFluidCollision):
    """Halfway bounce-back (boundary.hpp:14-31)."""
    kind = capi.LBM_NOSLIP

    def __init__(self, domain):
        super().__init__(domain)


class MovingWallBoundary(NonFluidCollision):
    """Bounce-back with wall velocity (boundary.hpp:43-68)."""
    kind = capi.LBM_MOVINGWALL

    def __init__(self, domain, wall_velocity):
        super().__init__(domain, wall_velocity)


class FreeSlipBoundary(NonFluidCollision):
    """Specular reflection (boundary.hpp:79-115)."""
    kind = capi.LBM_FREESLIP

    def __init__(self, domain):
        super().__init__(domain)


class OutflowBoundary(NonFluidCollision):
    """Anti-bounce-back at a reference density (boundary.hpp:128-150)."""
    kind = capi.LBM_OUTFLOW

    def __init__(self, domain, reference_density: float = 1.0):
        super().__init__(domain, rho=reference_density)


class InflowBoundary(NonFluidCollision):
    """Equilibrium at a given velocity (boundary.hpp:164-181)."""
    kind = capi.LBM_INFLOW

    def __init__(self, domain, inflow_velocity, reference_density: float = 1.0):
        super().__init__(domain, inflow_velocity, reference_density)

    def set_profile(self, u_cells: np.ndarray) -> None:
        """Extension: per-cell inflow velocity, array (Ng, 3) in reference cell order."""
        self.domain._set_inflow_profile(self.handler, u_cells)


class PressureBoundary(NonFluidCollision):
    """Anti-bounce-back at an imposed density (boundary.hpp:194-214)."""
    kind = capi.LBM_PRESSURE

    def __init__(self, domain, input_density: float):
        super().__init__(domain, rho=input_density)


class BoundaryKeeper:
    """BoundaryKeeper<M>::get_collision<BC>(args...) (boundary.h:72-91): creates a handler that
    lives as long as its domain."""

    @staticmethod
    def get_collision(cls, *args):
        return cls(*args)


class Domain:
    """Domain<M>(xl, yl, zl, collision, origin..., spacing...) (domain.h:22-26) on one GPU."""

    def __init__(self, xl: int, yl: int, zl: int, collision: FluidCollision, xorigin=0.0, yorigin=0.0,
                 zorigin=0.0, xspacing=1.0, yspacing=1.0, zspacing=1.0, model=_model.d3q19,
                 precision: str = "fp64"):
        self._lib = capi.load_library()
        self.model = _model.get(model)
        self.precision = precision
        self.xl, self.yl, self.zl = int(xl), int(yl), int(zl)
        self.xo, self.yo, self.zo = float(xorigin), float(yorigin), float(zorigin)
        self.xs, self.ys, self.zs = float(xspacing), float(yspacing), float(zspacing)
        self.collision = collision
        self._h = ctypes.c_void_p()
        rc = self._lib.lbm_create(ctypes.byref(self._h), self.model.Q, self.xl, self.yl, self.zl,
                                  collision.tau, capi.PRECISIONS[precision])
        if rc != capi.LBM_OK:
            raise LbmError(rc, self._lib.lbm_last_error(None).decode())
        self._phase = 0  # 0: idle, 1: stream() done, 2: swap() done
        self._handlers = []

    # -- lifetime ----------------------------------------------------------------------------
    def close(self) -> None:
        if self._h:
            self._lib.lbm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- getters (domain.h:28-36) ------------------------------------------------------------
    def xlength(self): return self.xl
    def ylength(self): return self.yl
    def zlength(self): return self.zl
    def xorigin(self): return self.xo
    def yorigin(self): return self.yo
    def zorigin(self): return self.zo
    def xspacing(self): return self.xs
    def yspacing(self): return self.ys
    def zspacing(self): return self.zs

    # -- helpers (domain.hpp:60-70) ----------------------------------------------------------
    def idx(self, x: int, y: int, z: int) -> int:
        return x + (self.xl + 2) * y + (self.xl + 2) * (self.yl + 2) * z

    def in_bounds(self, x: int, y: int, z: int) -> bool:
        return 0 < x < self.xl + 1 and 0 < y < self.yl + 1 and 0 < z < self.zl + 1

    @property
    def ncells(self) -> int:
        return (self.xl + 2) * (self.yl + 2) * (self.zl + 2)

    # -- geometry ------------------------------------------------------------------------------
    def _add_handler(self, kind: int, v, rho: float) -> int:
        params = (ctypes.c_double * 4)(v[0], v[1], v[2], rho)
        h = ctypes.c_int()
        check(self._lib.lbm_add_boundary(self._h, kind, params, ctypes.byref(h)), self._h)
        self._handlers.append(h.value)
        return h.value

    def setBoundaryCondition(self, condition: NonFluidCollision, x0, xE, y0, yE, z0, zE) -> None:
        """domain.hpp:174-194 (inclusive box, last writer wins)."""
        if condition.domain is not self:
            raise LbmError(capi.LBM_ERR_ARG, "boundary handler belongs to another domain")
        box = (ctypes.c_int64 * 6)(x0, xE, y0, yE, z0, zE)
        check(self._lib.lbm_set_boundary_box(self._h, condition.handler, box), self._h)

    def set_solid_mask(self, mask: np.ndarray) -> int:
        """Solid interior cells (mask shape (zl, yl, xl), nonzero = solid) bound to a new no-slip
        handler, as io::read_vtk_point_file does for mask value 0 (vtk.hpp:186-195)."""
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if m.size != self.xl * self.yl * self.zl:
            raise LbmError(capi.LBM_ERR_ARG, "mask size must be xl*yl*zl")
        h = ctypes.c_int()
        check(self._lib.lbm_set_solid_mask(self._h, m.ctypes.data, ctypes.byref(h)), self._h)
        self._handlers.append(h.value)
        return h.value

    def set_periodic(self, px: bool, py: bool, pz: bool) -> None:
        """Extension: periodic axes."""
        check(self._lib.lbm_set_periodic(self._h, int(px), int(py), int(pz)), self._h)

    def _set_inflow_profile(self, handler: int, u_cells) -> None:
        u = np.ascontiguousarray(u_cells, dtype=np.float64)
        if u.size != 3 * self.ncells:
            raise LbmError(capi.LBM_ERR_ARG, "profile must hold 3 values per cell")
        check(self._lib.lbm_set_inflow_profile(self._h, handler, u.ctypes.data), self._h)

    def set_nonfluid_cells_nullcollide(self) -> None:
        """domain.hpp:100-113 (result-neutral)."""
        check(self._lib.lbm_set_nonfluid_cells_nullcollide(self._h), self._h)

    # -- time loop (domain.hpp:115-172) --------------------------------------------------------
    def stream(self) -> None:
        if self._phase != 0:
            raise LbmError(capi.LBM_ERR_STATE, "stream() called twice without collide()")
        self._phase = 1

    def swap(self) -> None:
        if self._phase != 1:
            raise LbmError(capi.LBM_ERR_STATE, "swap() must follow stream()")
        self._phase = 2

    def collide(self) -> None:
        if self._phase != 2:
            raise LbmError(capi.LBM_ERR_STATE, "collide() must follow stream() and swap()")
        self._phase = 0
        self.step(1)

    def step(self, nsteps: int = 1) -> None:
        """nsteps x {stream(); swap(); collide();} in one call (asynchronous)."""
        check(self._lib.lbm_step(self._h, int(nsteps)), self._h)

    def step_monitored(self, nsteps: int, totals: np.ndarray | None = None) -> np.ndarray:
        """Extension: nsteps steps, each reporting the FP64 mass and momentum it started from
        (array (nsteps, 4)); valid after sync()."""
        out = totals if totals is not None else np.empty((int(nsteps), 4), dtype=np.float64)
        check(self._lib.lbm_step_monitored(self._h, int(nsteps), out.ctypes.data), self._h)
        self._monitor_keepalive = out
        return out

    def sync(self) -> None:
        check(self._lib.lbm_sync(self._h), self._h)

    @property
    def steps_done(self) -> int:
        return int(self._lib.lbm_steps_done(self._h))

    # -- inspection ----------------------------------------------------------------------------
    def populations(self) -> np.ndarray:
        """collide_field as an array (Ng, Q), reference cell order."""
        f = np.empty((self.ncells, self.model.Q), dtype=np.float64)
        check(self._lib.lbm_get_populations(self._h, f.ctypes.data), self._h)
        return f

    def set_populations(self, f: np.ndarray) -> None:
        a = np.ascontiguousarray(f, dtype=np.float64)
        if a.size != self.ncells * self.model.Q:
            raise LbmError(capi.LBM_ERR_ARG, "populations must be (Ng, Q)")
        check(self._lib.lbm_set_populations(self._h, a.ctypes.data), self._h)

    def cell(self, x: int, y: int, z: int) -> np.ndarray:
        """Populations of one cell (a copy; reads the whole field)."""
        return self.populations()[self.idx(x, y, z)]

    def moments(self):
        """(rho, u) of interior cells as arrays (zl, yl, xl) and (zl, yl, xl, 3)."""
        n = self.xl * self.yl * self.zl
        rho = np.empty(n, dtype=np.float64)
        u = np.empty(3 * n, dtype=np.float64)
        check(self._lib.lbm_moments(self._h, rho.ctypes.data, u.ctypes.data), self._h)
        return rho.reshape(self.zl, self.yl, self.xl), u.reshape(self.zl, self.yl, self.xl, 3)

    def reduce_mass_momentum(self) -> np.ndarray:
        out = np.empty(4, dtype=np.float64)
        check(self._lib.lbm_reduce_mass_momentum(self._h, out.ctypes.data), self._h)
        return out

    # -- gradients (extension) -------------------------------------------------------------
    def adjoint_forward(self, nsteps: int, ckpt_every: int) -> None:
        """nsteps steps from the current state, checkpointing every ckpt_every steps (1: every step's
        cell mass and momentum kept instead of state copies; the backward then recomputes nothing)."""
        check(self._lib.lbm_adjoint_forward(self._h, int(nsteps), int(ckpt_every)), self._h)

    def objective_ke(self, box) -> float:
        """sum over the fluid cells of box (x0, xE, y0, yE, z0, zE) of rho |u|^2 / 2."""
        b = (ctypes.c_int64 * 6)(*box)
        j = ctypes.c_double()
        check(self._lib.lbm_adjoint_objective_ke(self._h, b, ctypes.byref(j)), self._h)
        return j.value

    def adjoint_backward(self, box, dJ: float = 1.0):
        """(grad_inflow (Ng, 3), grad_wall (handlers, 3)) of objective_ke(box) at the end of the last
        adjoint_forward, times dJ."""
        b = (ctypes.c_int64 * 6)(*box)
        gin = np.zeros((self.ncells, 3), dtype=np.float64)
        n = len(self._handlers)
        gw = np.zeros((max(n, 1), 3), dtype=np.float64)  # row h - 1: handler id h
        check(self._lib.lbm_adjoint_backward(self._h, b, float(dJ), gin.ctypes.data, gw.ctypes.data), self._h)
        return gin, gw[:n]

    def stream_handle(self) -> int:
        s = ctypes.c_void_p()
        check(self._lib.lbm_get_stream(self._h, ctypes.byref(s)), self._h)
        return s.value or 0

    def memory_info(self):
        dev, step, fluid, launches = (ctypes.c_uint64() for _ in range(4))
        check(self._lib.lbm_memory_info(self._h, ctypes.byref(dev), ctypes.byref(step), ctypes.byref(fluid),
                                        ctypes.byref(launches)), self._h)
        return {"device_bytes": dev.value, "step_bytes": step.value, "fluid_cells": fluid.value,
                "launches_per_step": launches.value}
