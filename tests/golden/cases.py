"""Small parity cases shared by the fixture generator (make_golden.py) and the tests.

Each case is a Scenario plus a step count. Sizes are small and deliberately non-cubic so that an
axis mix-up cannot cancel out; together they exercise every boundary handler of the reference
(boundary.hpp), the three lattice models (model.h), last-writer-wins face edges (scenario.h),
interior solid cells, ghost cells left without a handler, and non-default initial populations.
"""
from __future__ import annotations

import numpy as np

from lbm_gb300 import scenario as S


def _shear(q):
    # shearflow.xml: pressure-driven channel with free-slip side walls
    s = S.Scenario("Shear", q, 8, 8, 20, 0.6)
    s.add_face("z0", "pressure", rho=1.005)
    s.add_face("zmax", "outflow")
    s.add_face("x0", "freeslip")
    s.add_face("xmax", "freeslip")
    s.add_face("y0", "noslip")
    s.add_face("ymax", "noslip")
    return s


def _step(q):
    # step.xml geometry at reduced size: inflow through part of z0, a solid block, outflow at zmax
    s = S.Scenario("Step", q, 12, 10, 16, 0.6)
    s.boundaries.append(S.Boundary("inflow", (7, 13, 0, 11, 0, 0), (0.0, 0.0, 0.05)))
    s.boundaries.append(S.Boundary("noslip", (0, 6, 0, 11, 0, 7)))
    s.add_face("zmax", "outflow")
    for f in ("y0", "ymax", "x0", "xmax"):
        s.add_face(f, "noslip")
    return s


def _ghost(q):
    # the README.xml example: three faces only, the other ghost cells stay fluid
    s = S.Scenario("Ghost", q, 9, 8, 10, 0.6)
    s.add_face("z0", "noslip")
    s.add_face("zmax", "movingwall", (0.05, 0.0, 0.0))
    s.add_face("ymax", "noslip")
    return s


def _random(q):
    s = S.cavity(10, q=q, ny=9, nz=8)
    s.solid = S.sphere_mask(10, 9, 8, (5, 5, 4), 2)
    rng = np.random.default_rng(7 + q)
    s.init = np.tile(s.model.weights, (s.ncells, 1)) * (1 + 0.05 * rng.standard_normal((s.ncells, q)))
    return s


def _channel(q):
    return S.channel(14, 10, 9, q=q, sphere=((7, 5, 5), 3))


CASES = {
    "cavity_q15": (lambda: S.cavity(10, q=15, ny=9, nz=8), 40),
    "cavity_q19": (lambda: S.cavity(10, q=19, ny=9, nz=8), 40),
    "cavity_q27": (lambda: S.cavity(10, q=27, ny=9, nz=8), 40),
    "channel_q15": (lambda: _channel(15), 30),
    "channel_q19": (lambda: _channel(19), 30),
    "channel_q27": (lambda: _channel(27), 30),
    "step_q19": (lambda: _step(19), 25),
    "shear_q15": (lambda: _shear(15), 30),
    "shear_q19": (lambda: _shear(19), 30),
    "shear_q27": (lambda: _shear(27), 30),
    "ghost_q19": (lambda: _ghost(19), 30),
    "ghost_q27": (lambda: _ghost(27), 30),
    "random_q19": (lambda: _random(19), 20),
    "random_q27": (lambda: _random(27), 20),
}

# Full-size FP64 cavity: 64^3 interior cells, tau 0.6, lid 0.05 on zmax, 1000 steps.
CAVITY64 = (lambda: S.cavity(64, q=19), 1000)
# Sample points kept in the cavity64 fixture (interior order index); the full field is pinned
# by a SHA-256 of its bytes.
CAVITY64_SAMPLE = np.arange(0, 64 ** 3, 61)
