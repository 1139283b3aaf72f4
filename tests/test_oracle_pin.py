"""Pins the CPU checkers (CPU only).

The C port (oracle/lbm_oracle.c) must reproduce the reference's own solver bit for bit: against
the committed fixtures in tests/golden (made by the reference build, see make_golden.py) and,
where the reference tree is present, against the reference compiled here.
"""
import hashlib

import numpy as np
import pytest

import oracle
from golden import cases
from lbm_gb300 import scenario as S
from lbm_gb300.model import C_S
from pathlib import Path

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_speed_of_sound_constant(oracle_built):
    # lbmdefinitions.h:47: 0.57735026919l as a double
    assert oracle.checkers.port_cs() == C_S
    assert C_S.hex() == "0x1.279a745904047p-1"
    if oracle.ref_available():
        assert oracle.checkers.ref_cs() == C_S


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_port_matches_golden_bit_exact(oracle_built, name):
    make, steps = cases.CASES[name]
    scn = make()
    g = np.load(GOLDEN / f"{name}.npz")
    assert int(g["steps"]) == steps
    r = oracle.run_port(scn, steps, threads=2)
    assert np.array_equal(r["pops"], g["pops"])
    assert np.array_equal(r["rho"], g["rho"])
    assert np.array_equal(r["u"], g["u"])


def test_port_cavity64_matches_golden_hash(oracle_built):
    make, steps = cases.CAVITY64
    g = np.load(GOLDEN / "cavity64_q19_1000.npz")
    r = oracle.run_port(make(), steps, threads=0)
    rho = r["rho"].reshape(-1)
    u = r["u"].reshape(-1, 3)
    assert hashlib.sha256(rho.tobytes()).hexdigest() == str(g["rho_sha256"])
    assert hashlib.sha256(u.tobytes()).hexdigest() == str(g["u_sha256"])
    idx = g["sample_index"]
    assert np.array_equal(rho[idx], g["rho"]) and np.array_equal(u[idx], g["u"])


def test_known_answer_cavity40():
    # Cavity D3Q19 40^3, tau 0.6, lid 0.05, 200 steps: rho and u_x at cell (20, 20, 40), as the
    # reference (built with FMA contraction) printed them: 0.99983949733793287,
    # 0.043240261119787557. Contraction changes the last bits only.
    r = oracle.run_port(S.cavity(40), 200, threads=0)
    rho = r["rho"][39, 19, 19]
    ux = r["u"][39, 19, 19, 0]
    assert abs(rho - 0.99983949733793287) < 1e-15
    assert abs(ux - 0.043240261119787557) < 1e-15 * 10


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present at build time")
@pytest.mark.parametrize("q", [15, 19, 27])
def test_port_matches_reference_build(oracle_built, q):
    # a case not in the fixtures: periodic-free channel with sphere and random initial state
    scn = S.channel(16, 11, 9, q=q, sphere=((8, 6, 5), 3))
    rng = np.random.default_rng(q)
    scn.init = np.tile(scn.model.weights, (scn.ncells, 1)) * (1 + 0.02 * rng.standard_normal((scn.ncells, q)))
    a = oracle.run_ref(scn, 17, threads=2)
    b = oracle.run_port(scn, 17, threads=2)
    assert np.array_equal(a["pops"], b["pops"])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present at build time")
def test_port_matches_reference_vtk_mask_quirk(oracle_built):
    # io::read_vtk_point_file marks solids in collide_field only (vtk.hpp:193-195); the port's
    # solid_mode 1 reproduces that as well
    scn = S.channel(20, 12, 12, q=19, sphere=((10, 6, 6), 3))
    a = oracle.run_ref(scn, 21, threads=2, solid_mode=1)
    b = oracle.run_port(scn, 21, threads=2, solid_mode=1)
    assert np.array_equal(a["pops"], b["pops"])
