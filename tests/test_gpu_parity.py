"""GPU parity: the CUDA step (through the C ABI) against the reference's solver.

FP64 storage must reproduce the reference bit for bit (same operations, same order, no fused
multiply-adds): populations, density and velocity compare with ==. The reference numbers come
from the committed fixtures (made by the reference's own headers, tests/golden/make_golden.py) and
from the C port of the reference (oracle/), which the CPU tests pin to those fixtures.
"""
import hashlib
from pathlib import Path

import numpy as np
import pytest

import oracle
from golden import cases
from helpers import defined_entries, rel_l2
from lbm_gb300 import LbmError, build_domain, capi
from lbm_gb300 import scenario as S

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _lib(lbm_lib, oracle_built):
    return lbm_lib


def _full_rows(mask, scn):
    """Interior cells whose every population is defined (for moment comparisons)."""
    rows = mask.reshape(scn.zl + 2, scn.yl + 2, scn.xl + 2, scn.q).all(axis=-1)
    return rows[1:-1, 1:-1, 1:-1]


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_fp64_bit_exact_vs_reference(name):
    make, steps = cases.CASES[name]
    scn = make()
    g = np.load(GOLDEN / f"{name}.npz")
    with build_domain(scn, "fp64") as dom:
        dom.step(steps)
        pops = dom.populations()
        rho, u = dom.moments()
    mask = defined_entries(scn)
    assert np.array_equal(pops[mask], g["pops"][mask])
    rows = _full_rows(mask, scn)
    assert np.array_equal(rho[rows], g["rho"][rows])
    assert np.array_equal(u[rows], g["u"][rows])


def test_fp64_cavity64_1000_steps_bit_exact():
    make, steps = cases.CAVITY64
    g = np.load(GOLDEN / "cavity64_q19_1000.npz")
    with build_domain(make(), "fp64") as dom:
        dom.step(steps)
        rho, u = dom.moments()
    rho = rho.reshape(-1)
    u = u.reshape(-1, 3)
    idx = g["sample_index"]
    assert np.array_equal(rho[idx], g["rho"])
    assert np.array_equal(u[idx], g["u"])
    assert hashlib.sha256(rho.tobytes()).hexdigest() == str(g["rho_sha256"])
    assert hashlib.sha256(u.tobytes()).hexdigest() == str(g["u_sha256"])


def test_time_loop_calls_equal_step():
    scn = S.cavity(12, q=19, ny=10, nz=9)
    with build_domain(scn) as a, build_domain(scn) as b:
        for _ in range(7):
            a.stream()
            a.swap()
            a.collide()
        b.step(7)
        assert a.steps_done == b.steps_done == 7
        assert np.array_equal(a.populations(), b.populations())


def test_time_loop_order_is_enforced():
    with build_domain(S.cavity(6)) as d:
        with pytest.raises(LbmError):
            d.collide()
        d.stream()
        with pytest.raises(LbmError):
            d.stream()


@pytest.mark.parametrize("q", [15, 19, 27])
@pytest.mark.parametrize("steps_before", [0, 3])
def test_populations_roundtrip_and_continue(q, steps_before):
    # set an arbitrary state at either layout parity, read it back, then keep stepping: the port
    # started from the same state must agree bit for bit
    scn = S.channel(13, 9, 8, q=q, sphere=((6, 5, 4), 2))
    rng = np.random.default_rng(100 + q)
    f0 = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.03 * rng.standard_normal((scn.ncells, q)))
    mask = defined_entries(scn)
    with build_domain(scn, "fp64") as dom:
        dom.step(steps_before)
        dom.set_populations(f0)
        back = dom.populations()
        assert np.array_equal(back[mask], f0[mask])
        dom.step(11)
        got = dom.populations()
    chk = oracle.Checker(scn)
    chk.set_populations(f0)
    chk.step(11)
    want = chk.populations()
    assert np.array_equal(got[mask], want[mask])


@pytest.mark.parametrize("q", [15, 19, 27])
def test_periodic_taylor_green_fp64_vs_port(q):
    scn = S.taylor_green(12, u0=0.05, omega=1.5, q=q)
    with build_domain(scn, "fp64") as dom:
        dom.step(23)
        rho, u = dom.moments()
    r = oracle.run_port(scn, 23)
    assert np.array_equal(rho, r["rho"]) and np.array_equal(u, r["u"])


def test_mixed_periodic_and_walls_fp64_vs_port():
    # periodic in x, walls elsewhere: wrapped pulls next to boundary cells
    scn = S.cavity(10, q=19, ny=7, nz=6)
    scn.boundaries = [b for b in scn.boundaries if b.extent[0] != b.extent[1] or b.extent[0] not in (0, 11)]
    scn.periodic = (True, False, False)
    with build_domain(scn, "fp64") as dom:
        dom.step(19)
        pops = dom.populations()
    want = oracle.run_port(scn, 19)["pops"]
    mask = defined_entries(scn)
    assert np.array_equal(pops[mask], want[mask])


def test_inflow_profile_fp64_vs_port():
    scn = S.adjoint_channel(16, 8, 7, omega=1.7)
    with build_domain(scn, "fp64") as dom:
        dom.step(21)
        pops = dom.populations()
    want = oracle.run_port(scn, 21)["pops"]
    mask = defined_entries(scn)
    assert np.array_equal(pops[mask], want[mask])


def test_geometry_change_mid_run_fp64_vs_port():
    scn = S.cavity(10, q=19, ny=9, nz=8)
    with build_domain(scn, "fp64") as dom:
        dom.step(9)
        from lbm_gb300 import BoundaryKeeper, NoSlipBoundary
        wall = BoundaryKeeper.get_collision(NoSlipBoundary, dom)
        dom.setBoundaryCondition(wall, 4, 6, 3, 5, 2, 4)
        dom.step(8)
        pops = dom.populations()
    chk = oracle.Checker(scn)
    chk.step(9)
    p = np.array([0, 0, 0, 1.0])
    hid = chk.lib.orc_add_boundary(chk.h, 1, p.ctypes.data)
    e = np.array([4, 6, 3, 5, 2, 4], dtype=np.int64)
    chk.lib.orc_set_boundary_box(chk.h, hid, e.ctypes.data)
    chk.step(8)
    want = chk.populations()
    scn2 = S.cavity(10, q=19, ny=9, nz=8)
    scn2.boundaries.append(S.Boundary("noslip", (4, 6, 3, 5, 2, 4)))
    mask = defined_entries(scn2)
    assert np.array_equal(pops[mask], want[mask])


def test_mass_momentum_reduction_matches_populations():
    scn = S.channel(20, 12, 11, q=19, sphere=((10, 6, 6), 3))
    with build_domain(scn, "fp64") as dom:
        dom.step(15)
        tot = dom.reduce_mass_momentum()
        pops = dom.populations()
    fluid = scn.fluid_mask_interior()
    f = pops.reshape(scn.zl + 2, scn.yl + 2, scn.xl + 2, scn.q)[1:-1, 1:-1, 1:-1][fluid]
    c = scn.model.velocities.astype(np.float64)
    want = np.array([f.sum(), (f @ c[:, 0]).sum(), (f @ c[:, 1]).sum(), (f @ c[:, 2]).sum()])
    assert abs(tot[0] - want[0]) <= 1e-12 * abs(want[0])
    assert np.allclose(tot[1:], want[1:], rtol=1e-10, atol=1e-12 * abs(want[0]))


def test_bad_arguments_on_device():
    with build_domain(S.cavity(6)) as d:
        from lbm_gb300 import BoundaryKeeper, NoSlipBoundary
        wall = BoundaryKeeper.get_collision(NoSlipBoundary, d)
        with pytest.raises(LbmError) as e:
            d.setBoundaryCondition(wall, 0, 8, 0, 0, 0, 0)  # xE = 8 > xl + 1
        assert e.value.code == capi.LBM_ERR_ARG
        with pytest.raises(LbmError):
            d.setBoundaryCondition(wall, 3, 2, 0, 0, 0, 0)  # end before begin
        with pytest.raises(LbmError):
            d.step(-1)


# ------------------------------------------------------------------------------------------
# Reduced precision: FP32 arithmetic on shifted FP32 / FP16 / BF16 storage against FP64.
# Tolerances: relative L2 over interior fluid cells, stated below.
# ------------------------------------------------------------------------------------------
TOL_U = {"fp32": 5e-6, "fp16": 2e-3, "bf16": 2e-2}
TOL_RHO = {"fp32": 2e-7, "fp16": 5e-5, "bf16": 5e-4}


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("q", [15, 19, 27])
def test_reduced_precision_channel(precision, q):
    scn = S.channel(32, 16, 16, q=q, sphere=((12, 8, 8), 4))
    steps = 200
    with build_domain(scn, "fp64") as d64:
        d64.step(steps)
        rho64, u64 = d64.moments()
    with build_domain(scn, precision) as d:
        d.step(steps)
        rho, u = d.moments()
    fl = scn.fluid_mask_interior()
    eu = rel_l2(u[fl], u64[fl])
    er = rel_l2(rho[fl] - 1.0, rho64[fl] - 1.0) * np.linalg.norm(rho64[fl] - 1) / np.linalg.norm(rho64[fl])
    print(f"{precision} q{q}: u rel L2 {eu:.3e}, rho rel L2 {er:.3e}")
    assert eu <= TOL_U[precision]
    assert er <= TOL_RHO[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("periodic", [False, True])
def test_step_monitor_matches_reduction(precision, periodic):
    # Every population a fluid cell pulls is some fluid cell's post-collision value (bounce-back
    # returns it to its own cell), so the mass a step starts from is the mass after the previous
    # step. Momentum too on a periodic box; walls reverse the momentum of bounced populations.
    if periodic:
        scn = S.taylor_green(12, u0=0.04, omega=1.6, q=19)
        scn.init = scn.init * (1 + 0.01 * np.random.default_rng(4).standard_normal(scn.init.shape))
    else:
        scn = S.cavity(14, q=19, lid=0.0, ny=11, nz=9)
        rng = np.random.default_rng(3)
        scn.init = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.02 * rng.standard_normal((scn.ncells, 19)))
    with build_domain(scn, precision) as dom:
        dom.step(5)
        before = dom.reduce_mass_momentum()
        tot = dom.step_monitored(3)
        dom.sync()
        after = dom.reduce_mass_momentum()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert abs(tot[0, 0] - before[0]) <= tol * before[0]
    assert abs(tot[2, 0] - tot[0, 0]) <= 10 * tol * before[0]
    assert abs(after[0] - tot[0, 0]) <= 10 * tol * before[0]
    if periodic:
        assert np.allclose(tot[0, 1:], before[1:], rtol=0, atol=10 * tol * before[0])


def test_step_monitor_counts_like_plain_steps():
    scn = S.channel(20, 10, 10, q=19, sphere=((8, 5, 5), 2))
    with build_domain(scn, "fp32") as a, build_domain(scn, "fp32") as b:
        a.step(12)
        b.step_monitored(12)
        b.sync()
        assert a.steps_done == b.steps_done == 12
        assert np.array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("box", ["closed", "periodic"])
def test_step_monitor_warp_sums_at_full_size(precision, box):
    # The step monitor sums the shifted moments of a warp's 32 cells in FP32 and adds the warp's
    # total to FP64 accumulators. On the 256 x 128 x 128 box that is 131,072 warps per step; the
    # bound asserted is 1e-7 absolute per warp (each warp sum rounds five times, at most 2^-24
    # of partial sums below 0.1). The comparison is exact in exact arithmetic: in a box closed by
    # no-slip walls every post-collision population is pulled exactly once by the next step
    # (bounce-back returns it to its own cell), so the mass the next step starts from is the mass
    # lbm_reduce_mass_momentum finds; on a periodic box the momentum too.
    xl, yl, zl = 256, 128, 128
    scn = S.Scenario("Box", 19, xl, yl, zl, 1.0 / 1.8)
    if box == "closed":
        for f in ("z0", "zmax", "x0", "xmax", "y0", "ymax"):
            scn.add_face(f, "noslip")
        scn.solid = S.sphere_mask(xl, yl, zl, (64, 64, 64), 16)
    else:
        scn.periodic = (True, True, True)
    rng = np.random.default_rng(11)
    scn.init = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.02 * rng.standard_normal((scn.ncells, 19)))
    warps = ((xl + 127) // 128) * yl * zl * 4
    bound = 1e-7 * warps
    with build_domain(scn, precision) as dom:
        dom.step(3)
        for _ in range(2):
            before = dom.reduce_mass_momentum()
            tot = dom.step_monitored(1)
            dom.sync()
            err = np.abs(tot[0] - before)
            print(f"{box} {precision}: mass error {err[0]:.3e}, momentum {err[1:].max():.3e} (bound {bound:.2e})")
            assert err[0] <= bound
            if box == "periodic":
                assert err[1:].max() <= bound


@pytest.mark.parametrize("steps_before", [0, 1])
def test_chunked_transfers_roundtrip_and_continue(steps_before):
    # 385 MB of FP64 D3Q27 populations: the upload and read-back go through the staging buffers
    # in a dozen chunks (at most 32 MiB each), alternating between the two buffers; an arbitrary
    # state set at either parity reads back unchanged and keeps stepping like the port started
    # from the same state
    scn = S.channel(200, 96, 88, q=27, sphere=((60, 48, 44), 12))
    rng = np.random.default_rng(21)
    f0 = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.03 * rng.standard_normal((scn.ncells, 27)))
    mask = defined_entries(scn)
    with build_domain(scn, "fp64") as dom:
        dom.step(steps_before)
        dom.set_populations(f0)
        back = dom.populations()
        assert np.array_equal(back[mask], f0[mask])
        dom.step(3)
        got = dom.populations()
        rho, u = dom.moments()
    chk = oracle.Checker(scn)
    chk.set_populations(f0)
    chk.step(3)
    want = chk.populations()
    wr, wu = chk.moments()
    chk.close()
    assert np.array_equal(got[mask], want[mask])
    fl = scn.fluid_mask_interior()
    assert np.array_equal(rho[fl], wr[fl]) and np.array_equal(u[fl], wu[fl])


@pytest.mark.parametrize("steps", [1, 2, 21])
def test_full_row_segments_fp64_vs_port(steps):
    # 256 cells along x with no-slip walls only: every 128-cell segment is made of bulk and wall
    # cells, so the step writes through the segment's shared-memory stage and row-wide bulk copies
    # (the unaligned ends of the odd steps' shifted rows directly); random initial populations
    scn = S.Scenario("Box", 19, 256, 9, 8, 0.6)
    for f in ("z0", "zmax", "x0", "xmax", "y0", "ymax"):
        scn.add_face(f, "noslip")
    rng = np.random.default_rng(31 + steps)
    scn.init = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.05 * rng.standard_normal((scn.ncells, 19)))
    with build_domain(scn, "fp64") as dom:
        dom.step(steps)
        pops = dom.populations()
    want = oracle.run_port(scn, steps)["pops"]
    mask = defined_entries(scn)
    assert np.array_equal(pops[mask], want[mask])


@pytest.mark.parametrize("q", [15, 27])
def test_full_row_segments_other_stencils(q):
    # the same with D3Q15 / D3Q27 in FP64 (bit for bit) and FP32 (against that FP64 run)
    scn = S.Scenario("Box", q, 256, 7, 6, 0.7)
    for f in ("z0", "zmax", "x0", "xmax", "y0", "ymax"):
        scn.add_face(f, "noslip")
    rng = np.random.default_rng(40 + q)
    scn.init = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.05 * rng.standard_normal((scn.ncells, q)))
    mask = defined_entries(scn)
    with build_domain(scn, "fp64") as dom:
        dom.step(9)
        p64 = dom.populations()
    assert np.array_equal(p64[mask], oracle.run_port(scn, 9)["pops"][mask])
    with build_domain(scn, "fp32") as dom:
        dom.step(9)
        p32 = dom.populations()
    assert np.abs(p32[mask] - p64[mask]).max() < 1e-6
