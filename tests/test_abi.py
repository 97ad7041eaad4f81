"""The C-ABI library loads and exports every function include/agx.h declares
(no device calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(agx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from anuga_core_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    names = declared("agx.h") + declared("agx_pool.h") + declared("agx_noalloc.h") + declared("agx_mesh.h")
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_footprint_and_version_without_device():
    from anuga_core_gb300 import _lib
    L = _lib.load()
    assert L.agx_version() >= 1
    assert _lib.footprint(1000, 40, 1520) > 1000 * 100
    assert _lib.footprint(2000, 40, 3020) > _lib.footprint(1000, 40, 1520)


def test_invalid_arguments_rejected_before_any_device_call():
    """The C ABI checks its arguments first: null handles and pointers, bad
    field ids and sizes come back as AGX_E_INVALID with a message, on a host
    without a GPU."""
    from anuga_core_gb300 import _lib, mixed
    INVALID = -1                                   # AGX_E_INVALID, include/agx.h
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.agx_scenario_create(None, None, ctypes.byref(h)) == INVALID
    assert "null" in _lib.last_error()
    buf = (ctypes.c_double * 4)()
    assert L.agx_get_field(None, 0, buf, 4) == INVALID
    assert "bad handle or field" in _lib.last_error()
    assert L.agx_set_field(None, 0, buf, 4) == INVALID
    assert L.agx_advance(None, 1, None) == INVALID
    assert "null handle" in _lib.last_error()
    P = mixed.lib()
    ph = ctypes.c_void_p()
    assert P.agx_pool_create(0, 0, 1, ctypes.byref(ph)) == INVALID
    assert P.agx_pool_create(1 << 31, 0, 1, ctypes.byref(ph)) == INVALID
