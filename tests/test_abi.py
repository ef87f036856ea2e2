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


def test_host_checks_before_any_device_call():
    """Argument mistakes are statuses, found before the library touches a
    device (these calls run without a GPU)."""
    lib = L.lib()
    assert lib.gfgpu_plan_create(None, None, None, None) == L.E_INVALID
    out = C.c_void_p()
    plans = (C.c_void_p * 2)(None, None)
    assert lib.gfgpu_batch_create(plans, 2, C.byref(out)) == L.E_INVALID
    assert b"null plan" in lib.gfgpu_last_error()
    assert lib.gfgpu_batch_create(None, 1, C.byref(out)) == L.E_INVALID
