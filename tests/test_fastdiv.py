"""Division by invariant integers (the step kernel's block-index decomposition), checked on the host
against plain division over the 32-bit range."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_fastdiv_matches_division(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    exe = tmp_path / "fastdiv_check"
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(ROOT / "lbm_gb300" / "csrc"), "-I", str(cuda_inc),
           str(ROOT / "tests" / "cpp" / "fastdiv_check.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "cuda_runtime.h" in r.stderr:
        pytest.skip("CUDA headers not found")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    assert " 0 wrong" in out.stdout
