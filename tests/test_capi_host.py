"""C ABI checks that need no GPU: the library loads, exports every entry point that
include/*.h declares, and validates arguments before touching the device."""
import ctypes
import re
from pathlib import Path

import pytest

from lbm_gb300 import capi

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared_functions():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(lbm_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "lbm_create" in names and "lbm_step" in names
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_library_exports_every_declared_symbol(lbm_lib):
    for name in declared_functions():
        assert hasattr(lbm_lib, name), name


def _create(lib, q=19, xl=8, yl=8, zl=8, tau=0.6, precision=capi.LBM_FP64):
    h = ctypes.c_void_p()
    rc = lib.lbm_create(ctypes.byref(h), q, xl, yl, zl, tau, precision)
    return rc, h


@pytest.mark.parametrize("kwargs,fragment", [
    (dict(q=18), "15, 19 or 27"),
    (dict(tau=0.5), "tau"),
    (dict(tau=2.0), "tau"),
    (dict(xl=0), "positive"),
    (dict(precision=7), "precision"),
    (dict(yl=70000), "too large"),
])
def test_create_rejects_bad_arguments(lbm_lib, kwargs, fragment):
    rc, h = _create(lbm_lib, **kwargs)
    assert rc == capi.LBM_ERR_ARG
    assert not h.value
    assert fragment in lbm_lib.lbm_last_error(None).decode()


def test_null_handle_is_an_argument_error(lbm_lib):
    assert lbm_lib.lbm_step(None, 1) == capi.LBM_ERR_ARG
    assert lbm_lib.lbm_sync(None) == capi.LBM_ERR_ARG
    assert lbm_lib.lbm_steps_done(None) == -1
    lbm_lib.lbm_destroy(None)
