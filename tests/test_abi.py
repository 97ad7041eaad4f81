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
