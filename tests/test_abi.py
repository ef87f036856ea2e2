"""The C-ABI library loads and exports every entry point include/gfgpu.h
declares (no device calls)."""
import ctypes as C
import os
import re

from getfem_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gfgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gfgpu_[a-z0-9_]+)\s*\(", src)))


def test_all_declared_symbols_exported():
    lib = C.CDLL(L.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) <= set(L.exported_symbols())


def test_version_and_error_text():
    lib = L.lib()
    assert b"sm_103a" in lib.gfgpu_version()
    assert lib.gfgpu_last_error() is not None
