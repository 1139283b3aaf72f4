"""The adjoint's BGK transpose (bgk_adjoint in adjoint.cuh, the moment form the adjoint step runs),
compiled for the host from the kernel source, against the transpose of a central-difference
Jacobian of the FP64 BGK map: D3Q15/19/27, FP64 and FP32, omega 0.6 .. 1.95."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_bgk_adjoint_matches_fd_jacobian(tmp_path):
    from lbm_gb300 import _build
    try:
        nvcc = _build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    if shutil.which(nvcc) is None and not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "bgk_adjoint_check"
    cmd = [nvcc, *_build.ARCH, "-std=c++17", "--expt-relaxed-constexpr", "-O2",
           "-I", str(ROOT / "lbm_gb300" / "csrc"), str(ROOT / "tests" / "cpp" / "bgk_adjoint_check.cu"),
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    assert out.stdout.count(" ok") == 3, out.stdout
