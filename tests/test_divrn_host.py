"""The FP64 step's correctly rounded division by precomputed reciprocal pairs (divrn.cuh), compiled
for the host from the kernel's own header, against IEEE division bit for bit; and the speed-of-sound
divisors' reciprocal pairs written in lattice.cuh against exact rational arithmetic."""
import os
import re
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import pytest

from lbm_gb300.model import C_S

ROOT = Path(__file__).resolve().parents[1]


def test_div_rn_matches_ieee_division(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    exe = tmp_path / "div_rn_check"
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(ROOT / "lbm_gb300" / "csrc"), "-I", str(cuda_inc),
           str(ROOT / "tests" / "cpp" / "div_rn_check.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "cuda_runtime.h" in r.stderr:
        pytest.skip("CUDA headers not found")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert " 0 wrong" in out.stdout


def test_speed_of_sound_reciprocal_pairs():
    # collision.hpp:45-46 divides by C_S*C_S, 2*C_S*C_S*C_S*C_S and 2*C_S*C_S, evaluated left to right
    divisors = {"cs2_div": C_S * C_S, "cs4x2_div": 2 * C_S * C_S * C_S * C_S, "cs2x2_div": 2 * C_S * C_S}
    text = (ROOT / "lbm_gb300" / "csrc" / "lattice.cuh").read_text()
    for name, y in divisors.items():
        m = re.search(name + r"\(\) \{ return \{(\w+), ([-0-9a-fx.p+]+), ([-0-9a-fx.p+]+)\}; \}", text)
        assert m, name
        zh, zl = float.fromhex(m.group(2)), float.fromhex(m.group(3))
        assert zh == 1.0 / y                                  # RN(1 / y)
        assert zl == float((1 - Fraction(y) * Fraction(zh)) / Fraction(y))  # RN((1 - y zh) / y)
