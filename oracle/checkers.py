"""TEST INFRASTRUCTURE ONLY: ctypes wrappers of the CPU checkers (see oracle/__init__.py)."""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
PORT_LIB = ORACLE_DIR / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libref_lbm.so"
REF_LIB_FAST = ORACLE_DIR / "_ref" / "libref_lbm_fast.so"


def reference_dir() -> Path | None:
    """The reference tree, named only by $LBM_REFERENCE_DIR (read at call time); None without it.
    Only building oracle/_ref and regenerating the fixtures read the reference."""
    d = os.environ.get("LBM_REFERENCE_DIR")
    return Path(d) if d else None


CONDITIONS = {"noslip": 1, "movingwall": 2, "freeslip": 3, "outflow": 4, "inflow": 5, "pressure": 6}


def build(with_ref: bool | None = None) -> None:
    """Compile the port (always) and the reference harness (when $LBM_REFERENCE_DIR names a
    reference tree)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "port"], check=True)
    ref = reference_dir()
    if with_ref is None:
        with_ref = ref is not None and (ref / "include" / "domain.hpp").exists()
    if with_ref:
        if ref is None:
            raise RuntimeError("LBM_REFERENCE_DIR is not set: the reference harness needs the reference tree")
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref", f"REF_DIR={ref}"], check=True)


def port_available() -> bool:
    return PORT_LIB.exists()


def ref_available() -> bool:
    return REF_LIB.exists()


_P = ctypes.c_void_p
_port = None
_ref = {}


def _load_port():
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build(with_ref=False)
        lib = ctypes.CDLL(str(PORT_LIB))
        lib.orc_create.restype = _P
        lib.orc_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double]
        lib.orc_destroy.argtypes = [_P]
        lib.orc_add_boundary.argtypes = [_P, ctypes.c_int, _P]
        lib.orc_set_boundary_box.argtypes = [_P, ctypes.c_int, _P]
        lib.orc_set_solid.argtypes = [_P, _P, ctypes.c_int]
        lib.orc_set_periodic.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.orc_set_inflow_profile.argtypes = [_P, ctypes.c_int, _P]
        lib.orc_set_populations.argtypes = [_P, _P]
        lib.orc_get_populations.argtypes = [_P, _P]
        lib.orc_step.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.orc_moments.argtypes = [_P, _P, _P]
        lib.orc_cs.restype = ctypes.c_double
        _port = lib
    return _port


def _load_ref(fast: bool = False):
    path = REF_LIB_FAST if fast else REF_LIB
    if path not in _ref:
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference tree at build time)")
        lib = ctypes.CDLL(str(path))
        lib.ref_run.restype = ctypes.c_int
        lib.ref_run.argtypes = ([ctypes.c_int] * 4 + [ctypes.c_double, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int,
                                                      _P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P])
        lib.ref_cs.restype = ctypes.c_double
        _ref[path] = lib
    return _ref[path]


def ref_cs() -> float:
    return _load_ref().ref_cs()


def port_cs() -> float:
    return _load_port().orc_cs()


class Checker:
    """The C port holding one scenario's state (two AoS fields, as the reference)."""

    def __init__(self, scn, solid_mode: int = 0):
        self.lib = _load_port()
        self.scn = scn
        self.Q = scn.q
        self.h = self.lib.orc_create(scn.q, scn.xl, scn.yl, scn.zl, scn.tau)
        if not self.h:
            raise RuntimeError("orc_create failed")
        if any(scn.periodic):
            self.lib.orc_set_periodic(self.h, *map(int, scn.periodic))
        if scn.solid is not None:
            m = np.ascontiguousarray(scn.solid, dtype=np.uint8)
            if self.lib.orc_set_solid(self.h, m.ctypes.data, solid_mode) < 0:
                raise RuntimeError("orc_set_solid failed")
        for b in scn.boundaries:
            p = np.array([*b.v, b.rho], dtype=np.float64)
            hid = self.lib.orc_add_boundary(self.h, CONDITIONS[b.condition], p.ctypes.data)
            if hid < 0:
                raise RuntimeError("orc_add_boundary failed")
            if b.profile is not None:
                prof = np.ascontiguousarray(b.profile, dtype=np.float64)
                self.lib.orc_set_inflow_profile(self.h, hid, prof.ctypes.data)
            e = np.array(b.extent, dtype=np.int64)
            if self.lib.orc_set_boundary_box(self.h, hid, e.ctypes.data) != 0:
                raise RuntimeError(f"bad extent {b.extent}")
        if scn.init is not None:
            self.set_populations(scn.init)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, n: int, threads: int = 0) -> float:
        sec = ctypes.c_double()
        self.lib.orc_step(self.h, int(n), int(threads), ctypes.byref(sec))
        return sec.value

    def populations(self) -> np.ndarray:
        f = np.empty((self.scn.ncells, self.Q), dtype=np.float64)
        self.lib.orc_get_populations(self.h, f.ctypes.data)
        return f

    def set_populations(self, f) -> None:
        a = np.ascontiguousarray(f, dtype=np.float64)
        self.lib.orc_set_populations(self.h, a.ctypes.data)

    def moments(self):
        n = self.scn.ninterior
        rho = np.empty(n)
        u = np.empty(3 * n)
        self.lib.orc_moments(self.h, rho.ctypes.data, u.ctypes.data)
        s = self.scn
        return rho.reshape(s.zl, s.yl, s.xl), u.reshape(s.zl, s.yl, s.xl, 3)


def run_port(scn, steps: int, threads: int = 0, solid_mode: int = 0) -> dict:
    c = Checker(scn, solid_mode)
    sec = c.step(steps, threads)
    rho, u = c.moments()
    out = {"pops": c.populations(), "rho": rho, "u": u, "seconds": sec}
    c.close()
    return out


def run_ref(scn, steps: int, threads: int = 0, solid_mode: int = 0, fast: bool = False,
            want_pops: bool = True) -> dict:
    """Run the reference's own Domain/BGKCollision/boundary code on the scenario."""
    if any(scn.periodic) or any(b.profile is not None for b in scn.boundaries):
        raise ValueError("the reference has no periodic axes or inflow profiles")
    lib = _load_ref(fast)
    t, p, e = scn.bc_arrays()
    t = np.ascontiguousarray(t)
    p = np.ascontiguousarray(p)
    e = np.ascontiguousarray(e)
    solid = None if scn.solid is None else np.ascontiguousarray(scn.solid, dtype=np.uint8)
    init = None if scn.init is None else np.ascontiguousarray(scn.init, dtype=np.float64)
    pops = np.empty((scn.ncells, scn.q)) if want_pops else None
    rho = np.empty(scn.ninterior)
    u = np.empty(3 * scn.ninterior)
    sec = ctypes.c_double()
    rc = lib.ref_run(scn.q, scn.xl, scn.yl, scn.zl, scn.tau, len(t), t.ctypes.data, p.ctypes.data, e.ctypes.data,
                     None if solid is None else solid.ctypes.data, solid_mode,
                     None if init is None else init.ctypes.data, steps, threads,
                     None if pops is None else pops.ctypes.data, rho.ctypes.data, u.ctypes.data, ctypes.byref(sec))
    if rc != 0:
        raise RuntimeError(f"ref_run failed ({rc})")
    return {"pops": pops, "rho": rho.reshape(scn.zl, scn.yl, scn.xl),
            "u": u.reshape(scn.zl, scn.yl, scn.xl, 3), "seconds": sec.value}
