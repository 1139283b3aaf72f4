"""Failure paths of the C ABI: the conditions the reference guards with asserts and exceptions
(configuration.h:123-128, domain.hpp:180-181) come back as status codes, and so do the device
conditions the reference cannot meet (divergence, device memory, a wait that gives up).

None of these faults, traps or hangs a GPU: the divergence is NaN arithmetic, the allocation
failure is a refused cudaMalloc, and the wait that gives up runs in a copy of the library built
with a poll limit of 0 for the row blocks' first wait, whose drain wait keeps its full limit.
"""
import ctypes
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

from lbm_gb300 import LbmError, build_domain, capi
from lbm_gb300 import scenario as S

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
def test_nan_populations_report_diverged(lbm_lib, precision):
    scn = S.channel(24, 12, 12, q=19, sphere=((8, 6, 6), 2))
    with build_domain(scn, precision) as dom:
        dom.step(2)
        assert np.all(np.isfinite(dom.reduce_mass_momentum()))
        f = dom.populations()
        f[dom.idx(12, 6, 6), 5] = np.nan
        dom.set_populations(f)
        dom.step(3)
        with pytest.raises(LbmError) as e:
            dom.reduce_mass_momentum()
        assert e.value.code == capi.LBM_ERR_DIVERGED
        assert "diverged" in str(e.value)
        tot = dom.step_monitored(2)  # the per-step totals carry the NaN as well
        dom.sync()
        assert not np.all(np.isfinite(tot))


def test_device_allocation_failure_reports_oom(lbm_lib):
    # D3Q27 FP64 with 2,139,103,232 cells (inside the 31-bit index limit): 462 GB of populations,
    # more than the GPU holds
    lib = lbm_lib
    h = ctypes.c_void_p(12345)
    rc = lib.lbm_create(ctypes.byref(h), 27, 2046, 1020, 1020, 0.6, capi.LBM_FP64)
    assert rc == capi.LBM_ERR_OOM
    assert h.value is None  # no handle is returned
    msg = lib.lbm_last_error(None).decode()
    assert "cudaMalloc(populations)" in msg
    # nothing of the refused allocation is left behind: a domain created next steps cleanly
    with build_domain(S.cavity(12, q=19), "fp32") as dom:
        dom.step(4)
        dom.sync()
        rho, _ = dom.moments()
        assert np.all(np.isfinite(rho))


_WAIT_SCRIPT = textwrap.dedent("""
    import ctypes, os, sys
    import numpy as np
    sys.path.insert(0, {root!r})
    from lbm_gb300 import LbmError, build_domain, capi
    from lbm_gb300 import scenario as S
    scn = S.channel(64, 32, 32, q=19, sphere=((20, 16, 16), 5))
    for prec in ("fp32", "fp64", "fp16"):
        with build_domain(scn, prec) as dom:
            dom.step(3)
            try:
                dom.sync()
            except LbmError as e:
                assert e.code == capi.LBM_ERR_CUDA, e
                assert "bounded wait" in str(e), e
            else:
                raise SystemExit("the give-up was not reported")
            # the error word is cleared and the context stays usable
            rho, u = dom.moments()
            assert np.all(np.isfinite(rho)) and np.all(np.isfinite(u))
            dom.sync()
    # the product library in the same process: a fresh handle steps cleanly
    capi._lib = None
    os.environ["LBM_GB300_LIBRARY"] = {product!r}
    with build_domain(scn, "fp32") as dom:
        dom.step(3)
        dom.sync()
        rho, _ = dom.moments()
        assert np.all(np.isfinite(rho))
    print("bounded-wait give-up reported")
""")


def test_row_wait_give_up_reports_cuda_error(lbm_lib, tmp_path):
    from lbm_gb300 import _build
    lib = _build.build(out_dir=tmp_path / "lib", defines=("LBMG_ROW_WAIT_POLLS=0u",))
    script = _WAIT_SCRIPT.format(root=str(ROOT), product=str(capi.library_path()))
    env = dict(os.environ, LBM_GB300_LIBRARY=str(lib))
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bounded-wait give-up reported" in r.stdout
