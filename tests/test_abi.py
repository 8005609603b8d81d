"""The C-ABI library builds, loads and exports every symbol include/*.h declares.

No compute call is made here (no GPU needed): only entry points whose
argument checks fail before touching CUDA are called.
"""

import ctypes
import glob
import os
import re

import pytest

from pyvr_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pvr_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pvr_render" in names and "pvr_create" in names and len(names) >= 10


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_abi_version(native_lib):
    assert native_lib.pvr_abi_version() == 1


def test_null_handle_errors(native_lib):
    lib = native_lib
    assert lib.pvr_destroy(None) == _native.PVR_OK
    lut = (ctypes.c_float * 4)(0, 0, 0, 0)
    assert lib.pvr_set_lut(None, lut, 1) == _native.PVR_ERR_VALUE
    assert b"null renderer" in lib.pvr_last_error()
    with pytest.raises(ValueError, match="null renderer"):
        _native.check(lib.pvr_set_config(None, 0.01, 10, 0.01))
    out = ctypes.c_void_p()
    assert lib.pvr_create(0, 5, ctypes.byref(out)) == _native.PVR_ERR_VALUE
    assert not out.value


def test_error_code_mapping():
    for code, exc in [(_native.PVR_ERR_VALUE, ValueError), (_native.PVR_ERR_TYPE, TypeError),
                      (_native.PVR_ERR_STATE, RuntimeError), (_native.PVR_ERR_NOMEM, MemoryError),
                      (_native.PVR_ERR_TIMEOUT, TimeoutError)]:
        with pytest.raises(exc):
            _native.check(code)
