"""The C++ drop-in interface (include/lbm_gb300.hpp): a program written against the reference's
API compiles against it, and on the GPU reproduces the reference's result bit for bit."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "cavity_drop_in.cpp"


@pytest.fixture(scope="module")
def drop_in_binary(lbm_lib, tmp_path_factory):
    from lbm_gb300 import _build
    exe = tmp_path_factory.mktemp("cpp") / "cavity_drop_in"
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
           "-L", str(_build.LIBDIR), "-llbm_gb300", f"-Wl,-rpath,{_build.LIBDIR}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_drop_in_program_compiles(drop_in_binary):
    assert drop_in_binary.exists()


@pytest.mark.gpu
def test_drop_in_program_matches_reference(drop_in_binary, tmp_path):
    g = np.load(ROOT / "tests" / "golden" / "cavity_q19.npz")
    out = tmp_path / "out.bin"
    res = subprocess.run([str(drop_in_binary), "10", "9", "8", str(int(g["steps"])), str(out)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    data = np.fromfile(out, dtype=np.float64)
    n = 10 * 9 * 8
    assert np.array_equal(data[:n], g["rho"].reshape(-1))
    assert np.array_equal(data[n:], g["u"].reshape(-1))
