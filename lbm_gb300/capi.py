"""ctypes binding of liblbm_gb300.so (the C ABI in include/lbm_gb300.h).

The library is built in-tree by ``lbm_gb300._build.build()``. Loading fails loudly when it is
missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from . import _build

# Status codes (include/lbm_gb300.h)
LBM_OK = 0
LBM_ERR_ARG = 1
LBM_ERR_OOM = 2
LBM_ERR_CUDA = 3
LBM_ERR_DIVERGED = 4
LBM_ERR_STATE = 5

# Boundary handler types
LBM_NOSLIP = 1
LBM_MOVINGWALL = 2
LBM_FREESLIP = 3
LBM_OUTFLOW = 4
LBM_INFLOW = 5
LBM_PRESSURE = 6

# Storage precisions
LBM_FP64 = 0
LBM_FP32 = 1
LBM_FP16 = 2
LBM_BF16 = 3
PRECISIONS = {"fp64": LBM_FP64, "fp32": LBM_FP32, "fp16": LBM_FP16, "bf16": LBM_BF16}
STORE_BYTES = {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}

_ERR_NAMES = {1: "LBM_ERR_ARG", 2: "LBM_ERR_OOM", 3: "LBM_ERR_CUDA", 4: "LBM_ERR_DIVERGED",
              5: "LBM_ERR_STATE"}

# name -> (restype, argtypes); every function include/lbm_gb300.h declares
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
SIGNATURES = {
    "lbm_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, _I64, _I64, _I64, _D, ctypes.c_int]),
    "lbm_destroy": (None, [_P]),
    "lbm_add_boundary": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.POINTER(ctypes.c_int)]),
    "lbm_set_boundary_box": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "lbm_set_solid_mask": (ctypes.c_int, [_P, _P, ctypes.POINTER(ctypes.c_int)]),
    "lbm_set_periodic": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "lbm_set_inflow_profile": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "lbm_set_nonfluid_cells_nullcollide": (ctypes.c_int, [_P]),
    "lbm_set_populations": (ctypes.c_int, [_P, _P]),
    "lbm_get_populations": (ctypes.c_int, [_P, _P]),
    "lbm_step": (ctypes.c_int, [_P, _I64]),
    "lbm_step_monitored": (ctypes.c_int, [_P, _I64, _P]),
    "lbm_moments": (ctypes.c_int, [_P, _P, _P]),
    "lbm_moments_noalloc": (ctypes.c_int, [_P, _P, _P]),
    "lbm_reduce_mass_momentum": (ctypes.c_int, [_P, _P]),
    "lbm_adjoint_forward": (ctypes.c_int, [_P, _I64, _I64]),
    "lbm_adjoint_objective_ke": (ctypes.c_int, [_P, _P, _P]),
    "lbm_adjoint_backward": (ctypes.c_int, [_P, _P, _D, _P, _P]),
    "lbm_sync": (ctypes.c_int, [_P]),
    "lbm_get_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "lbm_steps_done": (_I64, [_P]),
    "lbm_memory_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "lbm_last_error": (ctypes.c_char_p, [_P]),
}


class LbmError(RuntimeError):
    """A non-zero status from the C ABI; ``code`` is the LBM_ERR_* value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERR_NAMES.get(code, code)}: {message}")
        self.code = code


_lib = None


def library_path() -> Path:
    """liblbm_gb300.so in the package, or the file named by $LBM_GB300_LIBRARY."""
    env = os.environ.get("LBM_GB300_LIBRARY")
    return Path(env) if env else _build.LIB


def load_library(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load liblbm_gb300.so (optionally building it first) and declare every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with lbm_gb300._build.build() "
                               "(the CUDA step library has no CPU fallback)")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, handle=None) -> None:
    if rc != LBM_OK:
        lib = load_library()
        msg = lib.lbm_last_error(handle)
        raise LbmError(rc, msg.decode() if msg else "")
