"""Shifted FP32 / FP16 / BF16 storage against the reference's FP64 results, entry by entry, and the
headline channel at its full size.

The shifted path has boundary code of its own: a wall cell in a row block writes the values of
its moving-wall, inflow and outflow / pressure links from its LinkRecord (a handful of FP32
constants per cell), where the FP64 path evaluates the reference's handler formulas
(boundary.hpp:43-214). A wrong constant there would touch only the cells next to a boundary, so
these tests bound the largest error of the handler values themselves (the populations a
boundary cell holds for its fluid neighbours) and of the density and velocity of the cells next
to a boundary, not only a field-wide norm.

Tolerances (absolute, FP64 reference values as the truth; populations are O(0.3), the velocity
O(0.05)) are stated beside each test.
"""
import numpy as np
import pytest

import oracle
from golden import cases
from helpers import defined_entries, precision_errors, rel_l2
from lbm_gb300 import build_domain
from lbm_gb300 import scenario as S
from pathlib import Path

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _lib(lbm_lib, oracle_built):
    return lbm_lib


# Largest absolute error allowed after the golden cases' 20-40 steps: handler values and other
# populations / density and velocity. FP32 storage rounds s = f - w (|s| < 0.02) to 24 bits, so
# a single rounding is below 1e-9; FP16 to 11 bits (below 1e-5), BF16 to 8 bits (below 1e-4).
# Measured maxima over the 14 cases on GB300: FP32 1.3e-8 / 4.4e-8, FP16 2.1e-5 / 4.9e-5, BF16
# 1.8e-4 / 3.9e-4. A handler constant that is off by even the density's deviation from 1
# (about 1e-3 of a moving-wall term of 2e-2, 2e-5) is far outside the FP32 bounds.
TOL_GOLDEN = {
    "fp32": {"entries": 5e-8, "moments": 2e-7},
    "fp16": {"entries": 1e-4, "moments": 2e-4},
    "bf16": {"entries": 1e-3, "moments": 2e-3},
}


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_reduced_precision_golden_cases(name, precision):
    make, steps = cases.CASES[name]
    scn = make()
    g = np.load(GOLDEN / f"{name}.npz")
    with build_domain(scn, precision) as dom:
        dom.step(steps)
        pops = dom.populations()
        rho, u = dom.moments()
    e = precision_errors(scn, pops, rho, u, g["pops"], g["rho"], g["u"])
    tol = TOL_GOLDEN[precision]
    print(f"{name} {precision}: {e}")
    assert e["handler_entries"] <= tol["entries"], e
    assert e["fluid_entries"] <= tol["entries"], e
    assert max(e["u_linked"], e["u_bulk"], e["rho_linked"], e["rho_bulk"]) <= tol["moments"], e


# ------------------------------------------------------------------------------------------
# The headline configuration at full size: D3Q19 channel 256 x 128 x 128, inflow u_x 0.04 at
# x0, outflow rho 1 at xmax, no-slip walls, a solid sphere of radius 16 at (64, 64, 64),
# omega 1.8; 200 steps against the C port of the reference on all host cores.
# ------------------------------------------------------------------------------------------
HEADLINE_STEPS = 200
# relative L2 of u over the fluid cells, and the largest absolute errors (handler values, and
# density / velocity of the cells next to a boundary), after 200 steps. Measured on GB300:
# FP32 1.3e-6 / 9.8e-9 / 1.7e-7, FP16 3.4e-4 / 6.4e-6 / 4.2e-5.
TOL_HEADLINE = {
    "fp32": {"u_rel_l2": 5e-6, "entries": 5e-8, "moments": 1e-6},
    "fp16": {"u_rel_l2": 1e-3, "entries": 5e-5, "moments": 2e-4},
}


def headline_scenario():
    return S.channel(256, 128, 128, q=19, u_in=0.04, omega=1.8, sphere=((64, 64, 64), 16))


@pytest.fixture(scope="module")
def headline_port():
    scn = headline_scenario()
    r = oracle.run_port(scn, HEADLINE_STEPS)
    return scn, r


def test_headline_channel_full_size_fp64_bit_exact(headline_port):
    scn, want = headline_port
    with build_domain(scn, "fp64") as dom:
        dom.step(HEADLINE_STEPS)
        pops = dom.populations()
        rho, u = dom.moments()
    mask = defined_entries(scn)
    assert np.array_equal(pops[mask], want["pops"][mask])
    fl = scn.fluid_mask_interior()
    assert np.array_equal(rho[fl], want["rho"][fl])
    assert np.array_equal(u[fl], want["u"][fl])


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_headline_channel_full_size_reduced_precision(headline_port, precision):
    scn, want = headline_port
    with build_domain(scn, precision) as dom:
        dom.step(HEADLINE_STEPS)
        pops = dom.populations()
        rho, u = dom.moments()
    fl = scn.fluid_mask_interior()
    eu = rel_l2(u[fl], want["u"][fl])
    e = precision_errors(scn, pops, rho, u, want["pops"], want["rho"], want["u"])
    tol = TOL_HEADLINE[precision]
    print(f"headline {precision}: u rel L2 {eu:.3e} {e}")
    assert eu <= tol["u_rel_l2"], (eu, e)
    assert e["handler_entries"] <= tol["entries"], e
    assert max(e["u_linked"], e["rho_linked"]) <= tol["moments"], e


# ------------------------------------------------------------------------------------------
# The warp-shared handler path with LinkRecords: a moving wall on the x0 face (velocity in y and
# z) leaves one linked cell, x = 1, in the first warp of every inner row, so each of those warps
# hands that cell's moving-wall values (record constants times the cell's density) to the warp
# (FP32 with the record staged in shared memory, 16-bit storage reading it from global memory);
# the wall rows, every lane linked, take the per-lane path. 120 steps against the C port of the
# reference, per-cell maxima as in the headline test.
# ------------------------------------------------------------------------------------------
XLID_STEPS = 120
TOL_XLID = {  # the golden cases' bounds (entries for FP32 as the headline's)
    "fp32": {"entries": 5e-8, "moments": 1e-6},
    "fp16": {"entries": 1e-4, "moments": 2e-4},
    "bf16": {"entries": 1e-3, "moments": 2e-3},
}


def xlid_scenario(q):
    s = S.Scenario("XLid", q, 96, 32, 24, 0.6)
    for f in ("y0", "ymax", "z0", "zmax", "xmax"):
        s.add_face(f, "noslip")
    s.add_face("x0", "movingwall", (0.0, 0.05, -0.02))
    return s


@pytest.mark.parametrize("q", [19, 27])
def test_moving_wall_values_through_the_warp_shared_path(q):
    scn = xlid_scenario(q)
    want = oracle.run_port(scn, XLID_STEPS)
    for precision, tol in TOL_XLID.items():
        with build_domain(scn, precision) as dom:
            dom.step(XLID_STEPS)
            pops = dom.populations()
            rho, u = dom.moments()
        e = precision_errors(scn, pops, rho, u, want["pops"], want["rho"], want["u"])
        print(f"x-lid D3Q{q} {precision}: {e}")
        assert e["handler_entries"] <= tol["entries"], (precision, e)
        assert e["fluid_entries"] <= tol["entries"], (precision, e)
        assert max(e["u_linked"], e["rho_linked"], e["u_bulk"], e["rho_bulk"]) <= tol["moments"], (precision, e)


# ------------------------------------------------------------------------------------------
# A periodic box has no handler cells: its row blocks run the step kernel without the handler
# path (cells next to a wrap run in edge blocks). Taylor-Green 48^3, 100 steps, against the port.
# ------------------------------------------------------------------------------------------
TG_STEPS = 100
TOL_TG = {"fp32": {"entries": 1e-7, "moments": 1e-6},
          "fp16": {"entries": 1e-4, "moments": 2e-4},
          "bf16": {"entries": 1e-3, "moments": 2e-3}}


@pytest.mark.parametrize("q", [19, 27])
def test_periodic_box_reduced_precision(q):
    scn = S.taylor_green(48, u0=0.03, omega=1.7, q=q)
    want = oracle.run_port(scn, TG_STEPS)
    for precision, tol in TOL_TG.items():
        with build_domain(scn, precision) as dom:
            dom.step(TG_STEPS)
            pops = dom.populations()
            rho, u = dom.moments()
        e = precision_errors(scn, pops, rho, u, want["pops"], want["rho"], want["u"])
        fl = scn.fluid_mask_interior()
        eu = rel_l2(u[fl], want["u"][fl])
        print(f"Taylor-Green D3Q{q} {precision}: u rel L2 {eu:.3e} {e}")
        assert e["fluid_entries"] <= tol["entries"], (precision, e)
        assert max(e["u_bulk"], e["rho_bulk"]) <= tol["moments"], (precision, e)
