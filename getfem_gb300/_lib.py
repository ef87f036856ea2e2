"""ctypes binding of libgfgpu.so (the C ABI declared in include/gfgpu.h).

The shared library is built in-tree by getfem_gb300.build.  Loading fails
loudly when it is missing: there is no Python or CPU fallback for the
assembly kernels.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgfgpu.so")

OK, E_INVALID, E_UNSUPPORTED, E_CUDA, E_JACOBIAN, E_NAN, E_TIMEOUT, E_NOMEM, E_STATE = range(9)
SIMPLEX, HEX = 0, 1
COEF_NONE, COEF_CONST, COEF_ELEMENT, COEF_NODAL = 0, 1, 2, 3
TERM_GRADGRAD, TERM_MASS, TERM_SOURCE, TERM_NEOHOOKEAN, TERM_INTERNAL_P = 1, 2, 3, 4, 5
TERM_GRADGRAD_TENSOR = 6
MAX_TERMS = 8
MAX_TENSOR = 81
MAX_SLOTS = 8
SLOT_U = 0
REBUILD_PATTERN = 1
WITH_VECTOR = 2
PROFILE = 4
CONDENSATION = 8
SUM_FACTORISATION = 16
SLOT_POINTS = -1
RESULT_ROWPTR, RESULT_COLIDX, RESULT_VALUES, RESULT_VECTOR = 0, 1, 2, 3
RESULT_INTERNAL, RESULT_COUPLING, RESULT_COUPLING_COLIDX = 4, 5, 6

_STATUS_NAMES = {
    E_INVALID: "GFGPU_E_INVALID", E_UNSUPPORTED: "GFGPU_E_UNSUPPORTED", E_CUDA: "GFGPU_E_CUDA",
    E_JACOBIAN: "GFGPU_E_JACOBIAN", E_NAN: "GFGPU_E_NAN", E_TIMEOUT: "GFGPU_E_TIMEOUT",
    E_NOMEM: "GFGPU_E_NOMEM", E_STATE: "GFGPU_E_STATE",
}


class GfgpuError(RuntimeError):
    """Error raised for a nonzero gfgpu_status (the GMM_ASSERT1 analogue)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class UnsupportedExpression(GfgpuError):
    pass


class Coef(C.Structure):
    _fields_ = [("kind", C.c_int32), ("slot", C.c_int32), ("value", C.c_double)]


class Term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("field_slot", C.c_int32), ("scale", C.c_double),
                ("c", Coef * 3), ("aux_slot", C.c_int32), ("reserved", C.c_int32)]


class Form(C.Structure):
    _fields_ = [("n_terms", C.c_int32), ("terms", Term * MAX_TERMS),
                ("tensor", C.c_double * MAX_TENSOR)]


class Space(C.Structure):
    _fields_ = [("dim", C.c_int32), ("kind", C.c_int32), ("degree", C.c_int32),
                ("qdim", C.c_int32), ("im", C.c_char_p), ("n_points", C.c_int64),
                ("n_elements", C.c_int64), ("n_dof", C.c_int64),
                ("points", C.POINTER(C.c_double)), ("cvpts", C.POINTER(C.c_int64)),
                ("dofs", C.POINTER(C.c_int64))]


class Launch(C.Structure):
    """gfgpu_launch: threads per element of the element pass, warps per
    block of the row gather."""
    _fields_ = [("ep_threads", C.c_int32), ("gather_warps", C.c_int32)]


class NoallocArgs(C.Structure):
    _fields_ = [("dim", C.c_int32), ("degree", C.c_int32), ("qdim", C.c_int32),
                ("im", C.c_char_p), ("n_elements", C.c_int64), ("n_nodes", C.c_int64),
                ("points", C.c_void_p), ("cvpts", C.c_void_p), ("enode", C.c_void_p),
                ("adj_ptr", C.c_void_p), ("adj", C.c_void_p),
                ("slots", C.c_void_p * MAX_SLOTS), ("vec", C.c_void_p)]


NOALLOC_SCRATCH_BYTES = 128 << 20

_lib = None

# name -> (restype, argtypes)
_PROTOS = {
    "gfgpu_version": (C.c_char_p, []),
    "gfgpu_last_error": (C.c_char_p, []),
    "gfgpu_regular_unit_mesh": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                          C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.c_void_p, C.c_void_p]),
    "gfgpu_enumerate_dofs": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                       C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "gfgpu_enumerate_dofs_device": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int64, C.c_void_p, C.c_void_p,
                                              C.POINTER(C.c_int64)]),
    "gfgpu_device_available": (C.c_int, []),
    "gfgpu_nb_basis": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "gfgpu_quadrature": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.c_void_p, C.c_void_p]),
    "gfgpu_basis_tables": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_char_p,
                                     C.c_void_p, C.c_void_p]),
    "gfgpu_plan_create": (C.c_int, [C.POINTER(Space), C.POINTER(Form), C.c_void_p,
                                    C.POINTER(C.c_void_p)]),
    "gfgpu_plan_destroy": (None, [C.c_void_p]),
    "gfgpu_set_data": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_int32]),
    "gfgpu_pattern_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gfgpu_pattern_copy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfgpu_device_csr": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                   C.POINTER(C.c_void_p)]),
    "gfgpu_device_vector": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "gfgpu_assemble": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "gfgpu_assemble_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfgpu_assemble_host_upper": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfgpu_get_launch": (C.c_int, [C.c_void_p, C.POINTER(Launch)]),
    "gfgpu_set_launch": (C.c_int, [C.c_void_p, C.POINTER(Launch)]),
    "gfgpu_tune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Launch)]),
    "gfgpu_tune_save": (C.c_int, [C.c_char_p]),
    "gfgpu_tune_load": (C.c_int, [C.c_char_p]),
    "gfgpu_pattern_upper": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_void_p,
                                      C.c_void_p]),
    "gfgpu_sync": (C.c_int, [C.c_void_p]),
    "gfgpu_launch_count": (C.c_int64, [C.c_void_p]),
    "gfgpu_copy_result": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gfgpu_internal_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gfgpu_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    "gfgpu_fp64_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
    "gfgpu_assemble_vector_noalloc": (C.c_int, [C.POINTER(NoallocArgs), C.POINTER(Form),
                                                C.c_void_p]),
    "gfgpu_potential_gradient": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64,
                                           C.c_int32]),
    "gfgpu_set_points": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]),
    "gfgpu_dirichlet_eliminate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                            C.c_void_p]),
    "gfgpu_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "gfgpu_batch_assemble": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gfgpu_batch_tune": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32)]),
    "gfgpu_batch_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gfgpu_batch_elements": (C.c_int64, [C.c_void_p]),
    "gfgpu_batch_destroy": (None, [C.c_void_p]),
    "gfgpu_cg": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int64, C.c_int32,
                           C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
}


def exported_symbols() -> list[str]:
    return sorted(_PROTOS)


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: run getfem_gb300.build.build() "
                "(no CPU fallback exists for the assembly kernels)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        msg = lib().gfgpu_last_error().decode(errors="replace")
        if status == E_UNSUPPORTED:
            raise UnsupportedExpression(status, msg)
        raise GfgpuError(status, msg)
