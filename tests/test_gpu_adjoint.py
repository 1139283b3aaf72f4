"""Gradients by the discrete adjoint (an extension: the reference computes none) against FP64
central finite differences of the forward solver.

Objective: J = sum over the fluid cells of a box of rho |u|^2 / 2 after n steps. Parameters: the
per-cell inflow velocity profile (inflow handler) and a moving wall's velocity (lid). The FD
runs rebuild the domain with a perturbed parameter and repeat the same steps; the adjoint must
agree within 1e-4 relative (FP64 storage). FP32 and FP16 storage (FP32 arithmetic in the
adjoint) are compared with the FP64 gradient at the looser tolerances written below.
"""
import numpy as np
import pytest

from lbm_gb300 import BoundaryKeeper, LbmError, MovingWallBoundary, build_domain, capi
from lbm_gb300 import scenario as S
from helpers import rel_l2

pytestmark = pytest.mark.gpu
FD_RTOL = 1e-4


def _channel():
    # 20 x 10 x 8: inflow x0 (per-cell profile), outflow xmax, no-slip walls, 5 % solids
    return S.adjoint_channel(20, 10, 8, omega=1.7, seed=3)


def _cavity(lid=(0.05, 0.0, 0.0)):
    s = S.cavity(12, q=19, ny=10, nz=9, tau=0.6)
    s.boundaries[1].v = tuple(lid)
    return s


CH_BOX = (12, 19, 2, 9, 2, 7)
CAV_BOX = (3, 10, 2, 9, 5, 9)


def _objective(scn, steps, box, precision="fp64"):
    with build_domain(scn, precision) as d:
        d.step(steps)
        return d.objective_ke(box)


def _adjoint(scn, steps, ckpt, box, precision="fp64", pre=0):
    with build_domain(scn, precision) as d:
        d.step(pre)
        d.adjoint_forward(steps, ckpt)
        J = d.objective_ke(box)
        gin, gw = d.adjoint_backward(box)
        return J, gin, gw


def _inflow_index(scn, y, z):
    return (z * (scn.yl + 2) + y) * (scn.xl + 2)


def test_objective_matches_populations():
    scn = _channel()
    with build_domain(scn) as d:
        d.step(40)
        J = d.objective_ke(CH_BOX)
        rho, u = d.moments()
    x0, x1, y0, y1, z0, z1 = CH_BOX
    fl = scn.fluid_mask_interior()
    sl = (slice(z0 - 1, z1), slice(y0 - 1, y1), slice(x0 - 1, x1))
    r = rho[sl][fl[sl]]
    uu = (u[sl][fl[sl]] ** 2).sum(axis=-1)
    want = (0.5 * r * uu).sum()
    assert abs(J - want) <= 1e-12 * abs(want)


def test_adjoint_forward_equals_plain_steps():
    scn = _channel()
    with build_domain(scn) as a, build_domain(scn) as b:
        a.step(3)
        b.step(3)
        a.adjoint_forward(37, 8)
        b.step(37)
        assert a.steps_done == b.steps_done == 40
        assert np.array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("ckpt", [1, 16, 120])
def test_inflow_profile_gradient_vs_finite_differences(ckpt):
    scn = _channel()
    steps = 120
    J, gin, _ = _adjoint(scn, steps, ckpt, CH_BOX)
    assert J == _objective(scn, steps, CH_BOX)
    prof = scn.boundaries[0].profile
    h = 1e-5
    for (y, z, comp) in [(5, 4, 0), (2, 6, 0), (8, 3, 1), (4, 7, 2)]:
        k = _inflow_index(scn, y, z)
        vals = []
        for sgn in (1, -1):
            s2 = _channel()
            p2 = prof.copy()
            p2[k, comp] += sgn * h
            s2.boundaries[0].profile = p2
            vals.append(_objective(s2, steps, CH_BOX))
        fd = (vals[0] - vals[1]) / (2 * h)
        print(f"cell ({y},{z}) u{comp}: adjoint {gin[k, comp]:.9e} fd {fd:.9e}")
        assert abs(gin[k, comp] - fd) <= FD_RTOL * abs(fd) + 1e-9
    # nothing outside the inflow face
    face = np.zeros(scn.ncells, dtype=bool)
    for z in range(1, scn.zl + 1):
        for y in range(1, scn.yl + 1):
            face[_inflow_index(scn, y, z)] = True
    assert not np.any(gin[~face])


def test_inflow_directional_derivative_vs_finite_differences():
    # all inflow cells at once: d/de J(profile + e v) at e = 0 against sum(grad * v)
    scn = _channel()
    steps = 100
    _, gin, _ = _adjoint(scn, steps, 24, CH_BOX)
    rng = np.random.default_rng(11)
    v = np.zeros_like(scn.boundaries[0].profile)
    for z in range(1, scn.zl + 1):
        for y in range(1, scn.yl + 1):
            v[_inflow_index(scn, y, z)] = rng.standard_normal(3) * np.array([1.0, 0.3, 0.3])
    h = 1e-6
    vals = []
    for sgn in (1, -1):
        s2 = _channel()
        s2.boundaries[0].profile = s2.boundaries[0].profile + sgn * h * v
        vals.append(_objective(s2, steps, CH_BOX))
    fd = (vals[0] - vals[1]) / (2 * h)
    adj = float((gin * v).sum())
    print(f"directional: adjoint {adj:.9e} fd {fd:.9e}")
    assert abs(adj - fd) <= FD_RTOL * abs(fd)


@pytest.mark.parametrize("pre", [0, 7])
def test_lid_velocity_gradient_vs_finite_differences(pre):
    # pre > 0: the gradient run starts after `pre` plain steps and holds that state fixed,
    # including the lid values the previous step computed; the FD runs switch the lid to the
    # perturbed velocity at the same point (a new handler on the lid face)
    steps = 150
    lid = np.array([0.05, 0.0, 0.0])
    scn = _cavity(lid)
    J, _, gw = _adjoint(scn, steps, 32, CAV_BOX, pre=pre)
    g_lid = gw[1]  # handler 2: the zmax moving wall
    h = 1e-6
    fd = np.zeros(3)
    for comp in range(3):
        vals = []
        for sgn in (1, -1):
            v = lid.copy()
            v[comp] += sgn * h
            if pre == 0:
                vals.append(_objective(_cavity(v), steps, CAV_BOX))
            else:
                with build_domain(_cavity(lid)) as d:
                    d.step(pre)
                    w = BoundaryKeeper.get_collision(MovingWallBoundary, d, tuple(v))
                    # the lid cells only: the side walls applied after the lid own its edges
                    d.setBoundaryCondition(w, 1, scn.xl, 1, scn.yl, scn.zl + 1, scn.zl + 1)
                    d.step(steps)
                    vals.append(d.objective_ke(CAV_BOX))
        fd[comp] = (vals[0] - vals[1]) / (2 * h)
    print(f"lid gradient (pre {pre}): adjoint {g_lid} fd {fd}")
    scale = np.abs(fd).max()
    assert np.all(np.abs(g_lid - fd) <= FD_RTOL * np.abs(fd) + 1e-6 * scale)
    assert not np.any(gw[[0, 2, 3, 4, 5]])  # no-slip handlers carry no gradient


def test_pressure_outlet_gradient_vs_finite_differences():
    # pressure handler (rho-in 1.001) at xmax instead of the outflow one
    def make(delta=0.0):
        s = _channel()
        s.boundaries[1].condition = "pressure"
        s.boundaries[1].rho = 1.001
        s.boundaries[0].profile = s.boundaries[0].profile.copy()
        s.boundaries[0].profile[_inflow_index(s, 5, 4), 0] += delta
        return s
    steps = 90
    _, gin, _ = _adjoint(make(), steps, 30, CH_BOX)
    h = 1e-5
    fd = (_objective(make(h), steps, CH_BOX) - _objective(make(-h), steps, CH_BOX)) / (2 * h)
    g = gin[_inflow_index(make(), 5, 4), 0]
    print(f"pressure outlet: adjoint {g:.9e} fd {fd:.9e}")
    assert abs(g - fd) <= FD_RTOL * abs(fd)


@pytest.mark.parametrize("q", [15, 27])
def test_other_stencils_lid_gradient(q):
    steps = 80
    def make(v):
        s = S.cavity(10, q=q, ny=9, nz=8, tau=0.6)
        s.boundaries[1].v = tuple(v)
        return s
    box = (2, 9, 2, 8, 4, 8)
    _, _, gw = _adjoint(make((0.05, 0, 0)), steps, 20, box)
    h = 1e-6
    fd = (_objective(make((0.05 + h, 0, 0)), steps, box) - _objective(make((0.05 - h, 0, 0)), steps, box)) / (2 * h)
    print(f"D3Q{q} lid d/du_x: adjoint {gw[1, 0]:.9e} fd {fd:.9e}")
    assert abs(gw[1, 0] - fd) <= FD_RTOL * abs(fd)


# relative L2 of the reduced-precision gradient against the FP64 one
TOL_GRAD = {"fp32": 2e-5, "fp16": 2e-4, "bf16": 5e-3}


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_reduced_precision_gradients_vs_fp64(precision):
    scn = _channel()
    steps = 120
    _, g64, _ = _adjoint(scn, steps, 16, CH_BOX, "fp64")
    _, g, _ = _adjoint(scn, steps, 16, CH_BOX, precision)
    e = rel_l2(g, g64)
    print(f"{precision} inflow gradient rel L2 vs fp64: {e:.3e}")
    assert e <= TOL_GRAD[precision]
    cav = _cavity()
    _, _, w64 = _adjoint(cav, 150, 32, CAV_BOX, "fp64")
    _, _, w = _adjoint(cav, 150, 32, CAV_BOX, precision)
    e = rel_l2(w[1], w64[1])
    print(f"{precision} lid gradient rel L2 vs fp64: {e:.3e}")
    assert e <= TOL_GRAD[precision]


def test_backward_restores_state_and_can_repeat():
    scn = _channel()
    with build_domain(scn) as d:
        d.adjoint_forward(30, 7)
        before = d.populations()
        g1, _ = d.adjoint_backward(CH_BOX)
        assert np.array_equal(d.populations(), before)
        g2, _ = d.adjoint_backward(CH_BOX, dJ=2.0)
        # the gradients are sums of FP64 atomic adds (several cells and steps per inflow cell), whose
        # order follows the block scheduling, which the recompute stream running beside the adjoint
        # steps changes from call to call: equal to rounding, not bit for bit
        np.testing.assert_allclose(g2, 2.0 * g1, rtol=1e-12, atol=1e-15 * np.abs(g1).max())
        assert np.abs(g1).max() > 0
        assert d.steps_done == 30


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_resident_records_match_recompute(precision):
    # ckpt_every = 1 keeps every step's record from the forward: no recompute, the state is never
    # touched. Two handles in lockstep run the same forward steps with the two kinds of run in
    # turn, so each stage compares both on the same starting state (and the handle's workspace is
    # reallocated between the kinds). The adjoint is the same arithmetic on the same records; only
    # the order of the FP64 gradient atomics differs.
    scn = _channel()
    with build_domain(scn, precision) as a, build_domain(scn, precision) as b:
        for ka, kb in ((1, 13), (13, 1), (1, 7)):
            a.adjoint_forward(60, ka)
            b.adjoint_forward(60, kb)
            before = a.populations()
            assert np.array_equal(before, b.populations())
            ga, gwa = a.adjoint_backward(CH_BOX)
            gb, gwb = b.adjoint_backward(CH_BOX)
            assert np.array_equal(a.populations(), before)
            assert np.array_equal(b.populations(), before)
            scale = np.abs(gb).max()
            assert scale > 0
            np.testing.assert_allclose(ga, gb, rtol=0, atol=1e-12 * scale)
            ga2, _ = a.adjoint_backward(CH_BOX, dJ=2.0)  # repeatable with the kept records
            np.testing.assert_allclose(ga2, 2.0 * ga, rtol=0, atol=1e-12 * scale)
        assert a.steps_done == b.steps_done == 180


def test_resident_records_out_of_memory_is_reported():
    # records of 10^9 steps of the 20 x 10 x 8 channel (70 KB per step with the padded planes,
    # 70 TB in all) do not fit: a refused allocation, LBM_ERR_OOM, and the handle stays usable
    scn = _channel()
    with build_domain(scn, "fp32") as d:
        with pytest.raises(LbmError) as e:
            d.adjoint_forward(10**9, 1)
        assert e.value.code == capi.LBM_ERR_OOM
        assert "step records" in str(e.value)
        d.adjoint_forward(20, 1)
        g, _ = d.adjoint_backward(CH_BOX)
        assert np.all(np.isfinite(g))


def test_backward_needs_the_forward_state():
    scn = _channel()
    with build_domain(scn) as d:
        with pytest.raises(LbmError) as e:
            d.adjoint_backward(CH_BOX)
        assert e.value.code == capi.LBM_ERR_STATE
        d.adjoint_forward(5, 2)
        d.step(1)
        with pytest.raises(LbmError) as e:
            d.adjoint_backward(CH_BOX)
        assert e.value.code == capi.LBM_ERR_STATE
        with pytest.raises(LbmError) as e:
            d.objective_ke((0, 3, 1, 2, 1, 2))  # x0 = 0 is not interior
        assert e.value.code == capi.LBM_ERR_ARG


# ------------------------------------------------------------------------------------------
# the forward / backward contract wrapped as a torch.autograd.Function
# ------------------------------------------------------------------------------------------
def test_torch_autograd_function_wrapper():
    torch = pytest.importorskip("torch")

    class KineticEnergy(torch.autograd.Function):
        """J(inflow profile) = kinetic energy in a box after n steps; backward = the adjoint."""

        @staticmethod
        def forward(ctx, profile, steps, ckpt, box):
            scn = _channel()
            scn.boundaries[0].profile = profile.detach().cpu().numpy().astype(np.float64)
            dom = build_domain(scn, "fp64")
            dom.adjoint_forward(steps, ckpt)
            ctx.dom, ctx.box = dom, box
            return torch.tensor(dom.objective_ke(box), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            gin, _ = ctx.dom.adjoint_backward(ctx.box, dJ=float(grad_out))
            ctx.dom.close()
            return torch.from_numpy(gin), None, None, None

    prof = torch.tensor(_channel().boundaries[0].profile, requires_grad=True)
    J = KineticEnergy.apply(prof, 60, 16, CH_BOX)
    (g,) = torch.autograd.grad(3.0 * J, prof)
    # the same gradient as the C ABI call, scaled by the upstream factor (to rounding: the FP64
    # atomic adds of the gradient sums run in scheduling order)
    _, gin, _ = _adjoint(_channel(), 60, 16, CH_BOX)
    np.testing.assert_allclose(g.numpy(), 3.0 * gin, rtol=1e-12, atol=1e-15 * np.abs(gin).max())
    # and a directional finite difference through the wrapper itself
    v = torch.zeros_like(prof)
    k = _inflow_index(_channel(), 5, 4)
    v[k, 0] = 1.0
    h = 1e-5
    with torch.no_grad():
        jp = KineticEnergy.apply(prof + h * v, 60, 16, CH_BOX)
        jm = KineticEnergy.apply(prof - h * v, 60, 16, CH_BOX)
    fd = float(jp - jm) / (2 * h)
    assert abs(float((g * v).sum()) / 3.0 - fd) <= FD_RTOL * abs(fd)
