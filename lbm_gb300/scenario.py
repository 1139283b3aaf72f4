"""Scenarios: the reference's scenario description (domain size, boundaries in XML order,
solid cells) and the standard workloads built on it.

A Scenario is plain data, so the same description drives the GPU library (``build_domain``) and
the CPU checkers in tests. Named face extents follow io::parse_boundary (scenario.h:91-128):
each face covers the whole ghost plane, edges and corners included, and later boundaries
overwrite earlier ones cell by cell.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import capi
from . import model as _model

CONDITIONS = {
    "noslip": capi.LBM_NOSLIP,
    "movingwall": capi.LBM_MOVINGWALL,
    "freeslip": capi.LBM_FREESLIP,
    "outflow": capi.LBM_OUTFLOW,
    "inflow": capi.LBM_INFLOW,
    "pressure": capi.LBM_PRESSURE,
}


def face_extent(name: str, xl: int, yl: int, zl: int) -> tuple:
    """scenario.h:97-115"""
    faces = {
        "z0": (0, xl + 1, 0, yl + 1, 0, 0),
        "zmax": (0, xl + 1, 0, yl + 1, zl + 1, zl + 1),
        "x0": (0, 0, 0, yl + 1, 0, zl + 1),
        "xmax": (xl + 1, xl + 1, 0, yl + 1, 0, zl + 1),
        "y0": (0, xl + 1, 0, 0, 0, zl + 1),
        "ymax": (0, xl + 1, yl + 1, yl + 1, 0, zl + 1),
    }
    return faces[name]


@dataclass
class Boundary:
    condition: str                 # noslip | movingwall | freeslip | outflow | inflow | pressure
    extent: tuple                  # (x0, xE, y0, yE, z0, zE), inclusive
    v: tuple = (0.0, 0.0, 0.0)     # wall / inflow velocity
    rho: float = 1.0               # rho-ref (inflow, outflow) or rho-in (pressure)
    profile: np.ndarray | None = None  # extension: (Ng, 3) per-cell inflow velocity


@dataclass
class Scenario:
    name: str
    q: int
    xl: int
    yl: int
    zl: int
    tau: float
    boundaries: list = field(default_factory=list)
    solid: np.ndarray | None = None        # (zl, yl, xl) uint8, nonzero = solid no-slip
    periodic: tuple = (False, False, False)
    init: np.ndarray | None = None         # (Ng, Q) initial populations, or None for w_q
    origin: tuple = (0.0, 0.0, 0.0)
    spacing: tuple = (1.0, 1.0, 1.0)

    @property
    def model(self):
        return _model.get(self.q)

    @property
    def ncells(self) -> int:
        return (self.xl + 2) * (self.yl + 2) * (self.zl + 2)

    @property
    def ninterior(self) -> int:
        return self.xl * self.yl * self.zl

    def add_face(self, face: str, condition: str, v=(0.0, 0.0, 0.0), rho: float = 1.0) -> "Scenario":
        self.boundaries.append(Boundary(condition, face_extent(face, self.xl, self.yl, self.zl), tuple(v), rho))
        return self

    def bc_arrays(self):
        """(types int32[n], params float64[n,4], boxes int64[n,6]) in application order."""
        t = np.array([CONDITIONS[b.condition] for b in self.boundaries], dtype=np.int32)
        p = np.array([(*b.v, b.rho) for b in self.boundaries], dtype=np.float64).reshape(-1, 4)
        e = np.array([b.extent for b in self.boundaries], dtype=np.int64).reshape(-1, 6)
        return t, p, e

    def fluid_mask_interior(self) -> np.ndarray:
        """Interior cells that stay fluid after all boundaries and solids (zl, yl, xl) bool."""
        fl = np.ones((self.zl + 2, self.yl + 2, self.xl + 2), dtype=bool)
        for b in self.boundaries:
            x0, xe, y0, ye, z0, ze = b.extent
            fl[z0:ze + 1, y0:ye + 1, x0:xe + 1] = False
        inner = fl[1:-1, 1:-1, 1:-1].copy()
        if self.solid is not None:
            inner &= self.solid == 0
        return inner


def build_domain(scn: Scenario, precision: str = "fp64"):
    """Create a GPU Domain for the scenario through the reference-style API."""
    from .domain import (BGKCollision, BoundaryKeeper, Domain, FreeSlipBoundary, InflowBoundary,
                         MovingWallBoundary, NoSlipBoundary, OutflowBoundary, PressureBoundary)
    dom = Domain(scn.xl, scn.yl, scn.zl, BGKCollision(scn.tau), *scn.origin, *scn.spacing,
                 model=scn.q, precision=precision)
    if any(scn.periodic):
        dom.set_periodic(*scn.periodic)
    if scn.solid is not None:
        dom.set_solid_mask(scn.solid)
    for b in scn.boundaries:
        if b.condition == "noslip":
            h = BoundaryKeeper.get_collision(NoSlipBoundary, dom)
        elif b.condition == "movingwall":
            h = BoundaryKeeper.get_collision(MovingWallBoundary, dom, b.v)
        elif b.condition == "freeslip":
            h = BoundaryKeeper.get_collision(FreeSlipBoundary, dom)
        elif b.condition == "outflow":
            h = BoundaryKeeper.get_collision(OutflowBoundary, dom, b.rho)
        elif b.condition == "inflow":
            h = BoundaryKeeper.get_collision(InflowBoundary, dom, b.v, b.rho)
            if b.profile is not None:
                h.set_profile(b.profile)
        elif b.condition == "pressure":
            h = BoundaryKeeper.get_collision(PressureBoundary, dom, b.rho)
        else:
            raise ValueError(b.condition)
        dom.setBoundaryCondition(h, *b.extent)
    dom.set_nonfluid_cells_nullcollide()
    if scn.init is not None:
        dom.set_populations(scn.init)
    return dom


# ------------------------------------------------------------------------------------------
# Standard workloads
# ------------------------------------------------------------------------------------------
def cavity(n: int = 64, q: int = 19, lid: float = 0.05, tau: float = 0.6, ny: int | None = None,
           nz: int | None = None) -> Scenario:
    """Lid-driven cavity in the face order of cavity.xml: z0 noslip, zmax movingwall (lid, 0, 0),
    x0, xmax, y0, ymax noslip."""
    s = Scenario("Cavity", q, n, ny or n, nz or n, tau)
    s.add_face("z0", "noslip")
    s.add_face("zmax", "movingwall", (lid, 0.0, 0.0))
    for f in ("x0", "xmax", "y0", "ymax"):
        s.add_face(f, "noslip")
    return s


def sphere_mask(xl, yl, zl, center=(64, 64, 64), radius=16) -> np.ndarray:
    """Interior cells (1-based coordinates) with |x - center|^2 <= radius^2 -> 1."""
    z, y, x = np.meshgrid(np.arange(1, zl + 1), np.arange(1, yl + 1), np.arange(1, xl + 1), indexing="ij")
    d2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    return (d2 <= radius * radius).astype(np.uint8)


def channel(xl: int = 256, yl: int = 128, zl: int = 128, q: int = 19, u_in: float = 0.04,
            omega: float = 1.8, sphere=((64, 64, 64), 16)) -> Scenario:
    """Channel with a solid sphere, faces in the order of pipe.xml: z0, zmax noslip; x0 inflow
    (u_in, 0, 0) rho-ref 1; xmax outflow rho-ref 1; y0, ymax noslip."""
    s = Scenario("Channel", q, xl, yl, zl, 1.0 / omega)
    s.add_face("z0", "noslip")
    s.add_face("zmax", "noslip")
    s.add_face("x0", "inflow", (u_in, 0.0, 0.0), 1.0)
    s.add_face("xmax", "outflow", rho=1.0)
    s.add_face("y0", "noslip")
    s.add_face("ymax", "noslip")
    if sphere is not None:
        s.solid = sphere_mask(xl, yl, zl, *sphere)
    return s


def taylor_green(n: int = 384, u0: float = 0.03, omega: float = 1.9, q: int = 19) -> Scenario:
    """Decaying Taylor-Green vortex on a periodic box, started at f = feq(1, u_TG) with
    u = u0 (sin kx cos ky cos kz, -cos kx sin ky cos kz, 0), k = 2 pi / n."""
    s = Scenario("TaylorGreen", q, n, n, n, 1.0 / omega, periodic=(True, True, True))
    s.init = taylor_green_init(n, u0, q)
    return s


def taylor_green_velocity(n: int, u0: float, z_slab=None) -> np.ndarray:
    """u of the Taylor-Green vortex at the interior cells (z, y, x) (optionally only the z
    indices in z_slab), cell centres at (i + 1/2) k."""
    k = 2 * np.pi / n
    c = (np.arange(n) + 0.5) * k
    cz = c if z_slab is None else c[z_slab]
    z, y, x = np.meshgrid(cz, c, c, indexing="ij")
    u = np.empty(z.shape + (3,))
    u[..., 0] = u0 * np.sin(x) * np.cos(y) * np.cos(z)
    u[..., 1] = -u0 * np.cos(x) * np.sin(y) * np.cos(z)
    u[..., 2] = 0.0
    return u


def taylor_green_init(n: int, u0: float, q: int) -> np.ndarray:
    """(Ng, Q) populations: feq(1, u_TG) in the interior, w_q in the ghost layer; built one z
    slab at a time (the 384^3 box is 8.7 GB in FP64)."""
    m = _model.get(q)
    f = np.empty(((n + 2) ** 3, m.Q))
    f[:] = m.weights
    f4 = f.reshape(n + 2, n + 2, n + 2, m.Q)
    step = max(1, (1 << 22) // (n * n))
    for z0 in range(0, n, step):
        sl = slice(z0, min(n, z0 + step))
        u = taylor_green_velocity(n, u0, sl)
        f4[1 + sl.start:1 + sl.stop, 1:-1, 1:-1] = m.feq(np.ones(u.shape[:-1]), u)
    return f


def splitmix64(seed: int):
    """Deterministic generator shared with the C++ harness: splitmix64 -> uniform [0, 1)."""
    state = seed & 0xFFFFFFFFFFFFFFFF
    while True:
        state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        z = z ^ (z >> 31)
        yield (z >> 11) * (1.0 / (1 << 53))


def uniform(seed: int, n: int) -> np.ndarray:
    g = splitmix64(seed)
    return np.fromiter((next(g) for _ in range(n)), dtype=np.float64, count=n)


def adjoint_channel(xl: int = 128, yl: int = 64, zl: int = 64, omega: float = 1.7, q: int = 19,
                    seed: int = 0, solid_fraction: float = 0.05) -> Scenario:
    """Channel for the gradient workload: x0 inflow with a per-cell profile u_x ~ U[0.02, 0.05]
    over the yl x zl inlet, xmax outflow rho 1, then y0, ymax, z0, zmax noslip (so the walls own
    the inlet's edges), and a seeded 5 % of random solid cells kept off the x = 1 and x = xl
    planes."""
    s = Scenario("AdjointChannel", q, xl, yl, zl, 1.0 / omega)
    s.add_face("x0", "inflow", (0.035, 0.0, 0.0), 1.0)
    s.add_face("xmax", "outflow", rho=1.0)
    for f in ("y0", "ymax", "z0", "zmax"):
        s.add_face(f, "noslip")
    r = uniform(seed, yl * zl + xl * yl * zl)
    prof = np.zeros((zl + 2, yl + 2, xl + 2, 3))
    prof[1:-1, 1:-1, 0, 0] = 0.02 + 0.03 * r[: yl * zl].reshape(zl, yl)
    s.boundaries[0].profile = prof.reshape(-1, 3)
    solid = (r[yl * zl:].reshape(zl, yl, xl) < solid_fraction).astype(np.uint8)
    solid[:, :, 0] = 0
    solid[:, :, -1] = 0
    s.solid = solid
    return s
