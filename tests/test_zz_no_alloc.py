"""lbm_moments_noalloc, the moments read-back for callers that must not allocate device memory.

Some callers own all of their device memory through their own pool allocator, so a cudaMalloc
inside the library would fail once the pool holds the free memory (or would make the pool give
memory back); others read the moments every step, where a cudaMalloc / cudaFree pair per call
would synchronise the whole device. lbm_moments_noalloc serves them from a static device buffer
inside the library and must return exactly what lbm_moments returns.

This file sorts last so that a run stopping at the first failure has run every other test first;
it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from lbm_gb300 import BoundaryKeeper, LbmError, NoSlipBoundary, build_domain, capi
from lbm_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def _moments_noalloc(dom, with_u=True):
    n = dom.xl * dom.yl * dom.zl
    rho = np.empty(n, dtype=np.float64)
    u = np.empty(3 * n, dtype=np.float64) if with_u else None
    capi.check(dom._lib.lbm_moments_noalloc(dom._h, rho.ctypes.data, u.ctypes.data if with_u else None), dom._h)
    return rho, u


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_moments_match_lbm_moments(lbm_lib, precision):
    # the same kernel as lbm_moments on the same state: equal bit for bit
    scn = S.channel(40, 24, 20, q=19, sphere=((14, 12, 10), 4))
    with build_domain(scn, precision) as dom:
        for steps in (30, 7):
            dom.step(steps)
            rho_ref, u_ref = dom.moments()
            for _ in range(2):  # two calls in a row on the shared static buffer
                rho, u = _moments_noalloc(dom)
                assert np.array_equal(rho, rho_ref.reshape(-1))
                assert np.array_equal(u, u_ref.reshape(-1))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_density_only(lbm_lib, precision):
    # u may be NULL: only the density is computed and copied back
    scn = S.channel(40, 24, 20, q=19, sphere=((14, 12, 10), 4))
    with build_domain(scn, precision) as dom:
        dom.step(13)
        rho_ref, _ = dom.moments()
        for _ in range(2):
            rho, _ = _moments_noalloc(dom, with_u=False)
            assert np.array_equal(rho, rho_ref.reshape(-1))


def test_noalloc_rejects_domains_beyond_its_buffer(lbm_lib):
    # 65 x 64 x 64 = 266,240 interior cells > 262,144
    with build_domain(S.Scenario("Big", 19, 65, 64, 64, 0.6)) as dom:
        dom.step(1)
        with pytest.raises(LbmError) as e:
            _moments_noalloc(dom)
        assert e.value.code == capi.LBM_ERR_ARG
        assert "262144" in str(e.value)


def test_noalloc_needs_an_applied_geometry(lbm_lib):
    with build_domain(S.cavity(8)) as dom:
        dom.step(1)
        wall = BoundaryKeeper.get_collision(NoSlipBoundary, dom)
        dom.setBoundaryCondition(wall, 3, 4, 3, 4, 3, 4)
        with pytest.raises(LbmError) as e:
            _moments_noalloc(dom)
        assert e.value.code == capi.LBM_ERR_STATE
        dom.step(1)
        rho, _ = _moments_noalloc(dom)
        assert np.all(np.isfinite(rho))
