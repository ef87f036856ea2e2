"""getfem_gb300 — GB300-native backend for GetFEM's generic assembly hot path.

The package holds the host-side mirror of the reference interface
(GaWorkspace for ga_workspace, Mesh / MeshFem / MeshIm for the
discretisation objects, asm_generic for gf.asm('generic', ...)) over the
C ABI of libgfgpu.so (include/gfgpu.h), whose kernels run on sm_103a.
"""
from ._lib import GfgpuError, UnsupportedExpression  # noqa: F401
from .mesh import ImData, Mesh, MeshFem, MeshIm  # noqa: F401
from .workspace import GaWorkspace  # noqa: F401
from .adjoint import Potential  # noqa: F401
from . import solvers  # noqa: F401
from .asm import asm_generic  # noqa: F401

__all__ = ["GaWorkspace", "ImData", "Mesh", "MeshFem", "MeshIm", "Potential", "asm_generic",
           "GfgpuError", "UnsupportedExpression"]
