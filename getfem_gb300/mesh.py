"""Mesh, mesh_fem and mesh_im mirrors of GetFEM's discretisation objects.

Only what the assembly hot path reads is represented: node coordinates and
element->node connectivity (getfem::mesh), the per-element DOF map of a
Lagrange FEM with qdim components (getfem::mesh_fem,
mesh_fem::ind_scalar_basic_dof_of_element, getfem/getfem_mesh_fem.h:461) and
the integration method name (getfem::mesh_im).  Structured meshes and DOF
numbering come from the C ABI (gfgpu_regular_unit_mesh,
gfgpu_enumerate_dofs), which reproduce regular_unit_mesh and
mesh_fem::enumerate_dof exactly.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Mesh:
    """A conforming mesh of GT_PK(dim,1) simplices or GT_QK(dim,1) cubes."""

    def __init__(self, dim: int, kind: int, points: np.ndarray, cvpts: np.ndarray):
        self.dim = int(dim)
        self.kind = int(kind)
        self.points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, self.dim)
        nbpt = self.dim + 1 if self.kind == L.SIMPLEX else 2 ** self.dim
        self.cvpts = np.ascontiguousarray(cvpts, dtype=np.int64).reshape(-1, nbpt)

    @classmethod
    def regular_unit(cls, dim: int, nx: int, kind: str | int = "simplex", jitter=None) -> "Mesh":
        """getfem::regular_unit_mesh(m, {nx,..,nx}, GT_PK(dim,1) | GT_QK(dim,1)).

        jitter: optional (nx+1)^dim x dim array of offsets in lattice order
        (first index fastest), added to interior vertices."""
        k = L.SIMPLEX if kind in ("simplex", L.SIMPLEX) else L.HEX
        lib = L.lib()
        npt, ne = C.c_int64(), C.c_int64()
        L.check(lib.gfgpu_regular_unit_mesh(dim, k, nx, None, C.byref(npt), C.byref(ne), None, None))
        pts = np.empty((npt.value, dim))
        nbpt = dim + 1 if k == L.SIMPLEX else 2 ** dim
        cv = np.empty((ne.value, nbpt), dtype=np.int64)
        jp = None
        if jitter is not None:
            jitter = np.ascontiguousarray(jitter, dtype=np.float64)
            if jitter.size != (nx + 1) ** dim * dim:
                raise ValueError("jitter must hold (nx+1)^dim x dim values")
            jp = _ptr(jitter)
        L.check(lib.gfgpu_regular_unit_mesh(dim, k, nx, jp, C.byref(npt), C.byref(ne),
                                            _ptr(pts), _ptr(cv)))
        m = cls(dim, k, pts, cv)
        m.nx = nx
        return m

    def nb_points(self) -> int:
        return self.points.shape[0]

    def nb_convex(self) -> int:
        return self.cvpts.shape[0]


_FEM = re.compile(r"FEM_(PK|QK)\((\d+),(\d+)\)")


class MeshFem:
    """Lagrange FEM_PK/FEM_QK(dim, degree) on every convex, qdim components."""

    def __init__(self, mesh: Mesh, qdim: int = 1, fem: str | None = None, degree: int | None = None):
        self.mesh = mesh
        self.qdim = int(qdim)
        self.degree = None
        self.dofs = None
        if fem is not None:
            self.set_fem(fem)
        elif degree is not None:
            self.set_degree(degree)

    def set_fem(self, name: str) -> "MeshFem":
        m = _FEM.fullmatch(name.replace(" ", ""))
        if not m:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"FEM {name!r} is not supported")
        fam, dim, deg = m.group(1), int(m.group(2)), int(m.group(3))
        want = L.SIMPLEX if fam == "PK" else L.HEX
        if dim != self.mesh.dim or want != self.mesh.kind:
            raise ValueError(f"{name} does not match the mesh elements")
        return self.set_degree(deg)

    def set_degree(self, degree: int) -> "MeshFem":
        self.degree = int(degree)
        lib = L.lib()
        nb = C.c_int32()
        L.check(lib.gfgpu_nb_basis(self.mesh.dim, self.mesh.kind, self.degree, C.byref(nb)))
        self.nb = nb.value
        dofs = np.empty((self.mesh.nb_convex(), self.nb), dtype=np.int64)
        nd = C.c_int64()
        # the device numbering (a sort of node keys) where a GPU is visible
        # and the element fits its keys; the host numbering otherwise (the
        # two are identical, tests/test_gpu_dofs.py)
        on_dev = (self.degree >= 1 and self.degree <= 4 and lib.gfgpu_device_available()
                  and self.mesh.nb_points() < (1 << 25))
        enum = lib.gfgpu_enumerate_dofs_device if on_dev else lib.gfgpu_enumerate_dofs
        L.check(enum(self.mesh.dim, self.mesh.kind, self.degree, self.qdim,
                     self.mesh.nb_convex(), _ptr(self.mesh.cvpts), _ptr(dofs), C.byref(nd)))
        self.dofs = dofs
        self._nb_dof = nd.value
        return self

    def nb_dof(self) -> int:
        return self._nb_dof

    def fem_name(self) -> str:
        return f"FEM_{'PK' if self.mesh.kind == L.SIMPLEX else 'QK'}({self.mesh.dim},{self.degree})"

    def basic_dof_nodes(self) -> np.ndarray:
        """Coordinates of each DOF node (n_dof/qdim x dim), by the geometric
        transformation of each element's reference nodes."""
        from .refelem import lagrange_nodes, geo_basis
        ref = lagrange_nodes(self.mesh.dim, self.mesh.kind, self.degree)
        phi = geo_basis(self.mesh.dim, self.mesh.kind, ref)  # nb x nbg
        xyz = np.zeros((self._nb_dof // self.qdim, self.mesh.dim))
        X = self.mesh.points[self.mesh.cvpts]  # E x nbg x dim
        nodes = np.einsum("ig,egd->eid", phi, X)
        xyz[self.dofs // self.qdim] = nodes
        return xyz


class MeshIm:
    """An integration method on every convex (getfem::mesh_im)."""

    def __init__(self, mesh: Mesh, im: str):
        self.mesh = mesh
        self.im = im.replace(" ", "")
        lib = L.lib()
        d, nq = C.c_int32(), C.c_int32()
        L.check(lib.gfgpu_quadrature(self.im.encode(), C.byref(d), C.byref(nq), None, None))
        if d.value != mesh.dim:
            raise ValueError(f"{im} does not match the mesh dimension")
        self.nq = nq.value

    def points_weights(self):
        lib = L.lib()
        d, nq = C.c_int32(), C.c_int32()
        L.check(lib.gfgpu_quadrature(self.im.encode(), C.byref(d), C.byref(nq), None, None))
        pts = np.empty((nq.value, d.value))
        w = np.empty(nq.value)
        L.check(lib.gfgpu_quadrature(self.im.encode(), C.byref(d), C.byref(nq), _ptr(pts), _ptr(w)))
        return pts, w


class ImData:
    """Scalar data at the integration points of a mesh_im (getfem::im_data,
    getfem/getfem_im_data.h), one value per element Gauss point; point q of
    element e has index e * nq + q (im_data::index_of_point,
    src/getfem_im_data.cc:110-118, for a mesh_im over all convexes)."""

    def __init__(self, mim: MeshIm):
        self.mim = mim

    def nb_index(self) -> int:
        return self.mim.mesh.nb_convex() * self.mim.nq

    def nb_tensor_elem(self) -> int:
        return 1
