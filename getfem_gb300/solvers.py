"""Linear solves on the device from a workspace's assembled system.

Mirrors what a GetFEM user runs after assembly: boundary DOFs of the outer
faces (getfem::outer_faces_of_mesh + mesh_fem::dof_on_region), Dirichlet
conditions by elimination (the model's dof constraints,
getfem_models.cc:2806-2870) and gmm::cg (gmm/gmm_solver_cg.h) with the
identity or diagonal preconditioner.  The matrix is the plan's CSR on the
device; vectors are torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .refelem import lagrange_nodes


def _torch():
    import torch
    return torch


def _faces(dim: int, kind: int):
    """Local faces of the reference element as lists of geometric vertex
    indices, and the predicate selecting the reference nodes on face f."""
    if kind == L.SIMPLEX:
        nv = dim + 1
        faces = [[v for v in range(nv) if v != f] for f in range(nv)]

        def on(f, x):  # barycentric coordinate of vertex f vanishes
            lam = 1.0 - x.sum(axis=1) if f == 0 else x[:, f - 1]
            return np.abs(lam) < 1e-12
        return faces, on
    faces, preds = [], []
    for d in range(dim):
        for side in (0, 1):
            faces.append([p for p in range(2 ** dim) if ((p >> d) & 1) == side])
            preds.append((d, side))

    def on(f, x):
        d, side = preds[f]
        return np.abs(x[:, d] - side) < 1e-12
    return faces, on


def boundary_dofs(mf) -> np.ndarray:
    """DOFs of mf on the outer faces of its mesh (faces of exactly one
    element), all qdim components, sorted: mf.dof_on_region of the region
    built by getfem::outer_faces_of_mesh."""
    m = mf.mesh
    faces, on = _faces(m.dim, m.kind)
    keys = {}
    for e in range(m.nb_convex()):
        cv = m.cvpts[e]
        for f, fv in enumerate(faces):
            k = tuple(sorted(int(cv[v]) for v in fv))
            keys.setdefault(k, []).append((e, f))
    ref = lagrange_nodes(m.dim, m.kind, mf.degree)
    local = [np.nonzero(on(f, ref))[0] for f in range(len(faces))]
    out = set()
    for occ in keys.values():
        if len(occ) != 1:
            continue
        e, f = occ[0]
        for li in local[f]:
            base = int(mf.dofs[e, li])
            for a in range(mf.qdim):
                out.add(base + a)
    return np.array(sorted(out), dtype=np.int64)


def dirichlet_eliminate(plan, dofs, values=None, rhs=None):
    """Eliminates the constrained DOFs from the plan's assembled K (and
    adjusts rhs, a torch CUDA tensor, in place)."""
    d = np.ascontiguousarray(np.asarray(dofs, dtype=np.int64))
    v = None if values is None else np.ascontiguousarray(np.asarray(values, dtype=np.float64))
    if v is not None and v.size != d.size:
        raise ValueError("one value per constrained DOF")
    L.check(L.lib().gfgpu_dirichlet_eliminate(
        plan, d.ctypes.data_as(C.c_void_p), d.size,
        None if v is None else v.ctypes.data_as(C.c_void_p),
        None if rhs is None else C.c_void_p(rhs.data_ptr())))


def cg(plan, b, x=None, resmax: float = 1e-12, maxiter: int = 100000,
       precond: str = "identity"):
    """gmm::cg on the plan's K: returns (x, iterations, relative residual)."""
    torch = _torch()
    b = b.contiguous()
    x = torch.zeros_like(b) if x is None else x.contiguous()
    it, res = C.c_int64(), C.c_double()
    pc = {"identity": 0, "diagonal": 1, "jacobi": 1}[precond]
    L.check(L.lib().gfgpu_cg(plan, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                             float(resmax), int(maxiter), pc, C.byref(it), C.byref(res)))
    return x, it.value, res.value


def solve_linear(ws, dirichlet_dofs, dirichlet_values=None, resmax: float = 1e-12,
                 maxiter: int = 100000, precond: str = "identity", group: int = 0):
    """Solves the workspace's linear problem K du = -R(u) for its variable u
    with Dirichlet conditions u(D) = values (zero by default), on the device:
    order-2 and order-1 assemblies, elimination, CG.  Returns (u, info)."""
    torch = _torch()
    g = ws.groups[group]
    lib = L.lib()
    h2 = ws._plan(g, g.order2)
    h1 = ws._plan(g, g.order1)
    u0 = g.var.values
    ws._upload(h2, g.order2, need_u=False)
    ws._upload(h1, g.order1, need_u=True)
    L.check(lib.gfgpu_assemble(h2, 2, 0, None))
    L.check(lib.gfgpu_assemble(h1, 1, 0, None))
    n = g.var.mf.nb_dof()
    rhs = torch.empty(n, dtype=torch.float64, device="cuda")
    L.check(lib.gfgpu_copy_result(h1, L.RESULT_VECTOR, C.c_void_p(rhs.data_ptr())))
    rhs.neg_()
    u0t = torch.as_tensor(np.asarray(u0, dtype=np.float64)).to("cuda") \
        if not hasattr(u0, "is_cuda") else u0.to(torch.float64)
    d = np.asarray(dirichlet_dofs, dtype=np.int64)
    gv = np.zeros(d.size) if dirichlet_values is None else np.asarray(dirichlet_values, float)
    du_d = gv - u0t[torch.as_tensor(d, device="cuda")].cpu().numpy()
    dirichlet_eliminate(h2, d, du_d, rhs)
    du, it, res = cg(h2, rhs, None, resmax, maxiter, precond)
    return u0t + du, {"iterations": it, "residual": res}
