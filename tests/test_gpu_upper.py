"""The symmetric-matrix host delivery (gfgpu_assemble_host_upper): the upper
triangle of K (entries with column >= row) copied to host memory, half of
the values.  Mirroring it must give the full K exactly, so K has to be
symmetric bit for bit on every element-kernel family (affine simplices,
Gauss-point hexahedra with the neo-Hookean tangent, parallelepiped
hexahedra); the upper values must equal those of the full host delivery
bit for bit, on the first call (pattern build) and on later calls (chunked
copies overlapping the gather)."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import getfem_gb300 as g
from getfem_gb300 import _lib as L

pytestmark = pytest.mark.gpu

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"


def _case(name):
    rng = np.random.default_rng(11)
    if name == "p2tet_elastic":
        nx = 4
        h = 1.0 / nx
        jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
        mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
        mf = g.MeshFem(mesh, 3, degree=2)
        mim = g.MeshIm(mesh, "IM_TETRAHEDRON(5)")
        mf0 = g.MeshFem(mesh, 1, degree=0)
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 1e-3)
        ws.add_fem_constant("lambda", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        ws.add_fem_constant("mu", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        ws.add_fem_constant("f", mf, rng.standard_normal(mf.nb_dof()))
        ws.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u", mim)
    elif name == "p2tri_poisson":
        mesh = g.Mesh.regular_unit(2, 6, "simplex")
        mf = g.MeshFem(mesh, 1, degree=2)
        mim = g.MeshIm(mesh, "IM_TRIANGLE(4)")
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()))
        ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        ws.add_expression("kappa*Grad_u.Grad_Test_u + 2*u*Test_u", mim)
    elif name == "q2hex_neohookean":
        mesh = g.Mesh.regular_unit(3, 2, "hex")
        mf = g.MeshFem(mesh, 3, degree=2)
        mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
        xyz = mf.basic_dof_nodes()
        u = 0.05 * np.sin(xyz @ rng.uniform(-3, 3, (3, 3)))
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=u.ravel())
        ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.3, mesh.nb_convex())))
        ws.add_fixed_size_constant("D1", np.array([1.5]))
        ws.add_expression(NH, mim)
    elif name == "q4hex_laplace":
        mesh = g.Mesh.regular_unit(3, 2, "hex")
        mf = g.MeshFem(mesh, 1, degree=4)
        mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,9)")
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()))
        ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.5, mesh.nb_convex())))
        ws.add_expression("kappa*Grad_u.Grad_Test_u", mim)
    else:
        raise KeyError(name)
    return mesh, mf, ws


def _plan(ws):
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1)
    ws._upload(h, grp.order1, need_u=True)
    return h


def _upper(h, n, u, nnz_upper=None):
    """Two calls of gfgpu_assemble_host_upper and the upper pattern.  With
    nnz_upper given, the plan is fresh (its first call builds the pattern)."""
    lib = L.lib()
    nnz_u = C.c_int64(nnz_upper if nnz_upper is not None else 0)
    if nnz_upper is None:
        L.check(lib.gfgpu_pattern_upper(h, C.byref(nnz_u), None, None))
    out, vecs = [], []
    for _ in range(2):
        vec = np.empty(n)
        uv = np.empty(nnz_u.value)
        L.check(lib.gfgpu_assemble_host_upper(h, u.ctypes.data, uv.ctypes.data, vec.ctypes.data))
        out.append(uv)
        vecs.append(vec)
    rowptr = np.empty(n + 1, dtype=np.int64)
    colidx = np.empty(nnz_u.value, dtype=np.int32)
    L.check(lib.gfgpu_pattern_upper(h, C.byref(nnz_u), rowptr.ctypes.data, colidx.ctypes.data))
    return rowptr, colidx, out, vecs


@pytest.mark.parametrize("name", ["p2tet_elastic", "p2tri_poisson", "q2hex_neohookean",
                                  "q4hex_laplace"])
def test_upper_triangle_is_the_full_matrix(name):
    mesh, mf, ws = _case(name)
    n = mf.nb_dof()
    h = _plan(ws)
    lib = L.lib()
    u = np.ascontiguousarray(ws.data["u"].values, dtype=np.float64)
    vec_full = np.empty(n)
    L.check(lib.gfgpu_assemble_host(h, u.ctypes.data, None, vec_full.ctypes.data))
    nr, nnz = C.c_int64(), C.c_int64()
    L.check(lib.gfgpu_pattern_size(h, C.byref(nr), C.byref(nnz)))
    rp = np.empty(n + 1, dtype=np.int64)
    ci = np.empty(nnz.value, dtype=np.int32)
    L.check(lib.gfgpu_pattern_copy(h, rp.ctypes.data, ci.ctypes.data))
    vals = np.empty(nnz.value)
    L.check(lib.gfgpu_assemble_host(h, u.ctypes.data, vals.ctypes.data, vec_full.ctypes.data))
    K = sp.csr_matrix((vals, ci, rp), shape=(n, n))
    # symmetric bit for bit: same pattern and the same values transposed
    KT = K.T.tocsr()
    KT.sort_indices()
    assert np.array_equal(KT.indptr, K.indptr) and np.array_equal(KT.indices, K.indices)
    assert np.array_equal(KT.data, K.data)
    rowptr, colidx, uvals, vecs = _upper(h, n, u)
    U = sp.triu(K, format="csr")
    U.sort_indices()
    assert np.array_equal(rowptr, U.indptr) and np.array_equal(colidx, U.indices)
    for uv, vec in zip(uvals, vecs):
        assert np.array_equal(uv, U.data)
        assert np.array_equal(vec, vec_full)
    # a fresh plan whose first call is the upper delivery
    _, mf2, ws2 = _case(name)
    r2, c2, uv2, v2 = _upper(_plan(ws2), n, u, nnz_upper=U.nnz)
    assert np.array_equal(r2, U.indptr) and np.array_equal(c2, U.indices)
    for uv, vec in zip(uv2, v2):
        assert np.array_equal(uv, U.data)
        assert np.array_equal(vec, vec_full)
    # mirroring the upper values rebuilds K exactly
    Ku = sp.csr_matrix((uvals[-1], colidx, rowptr), shape=(n, n))
    M = (Ku + sp.triu(Ku, k=1).T).tocsr()
    M.sort_indices()
    assert np.array_equal(M.indptr, K.indptr) and np.array_equal(M.indices, K.indices)
    assert np.array_equal(M.data, K.data)


def test_upper_refused_for_a_nonsymmetric_form():
    rng = np.random.default_rng(2)
    mesh = g.Mesh.regular_unit(3, 2, "hex")
    mf = g.MeshFem(mesh, 3, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.05)
    ws.add_internal_im_variable("p", g.ImData(mim), rng.standard_normal(mesh.nb_convex() * 27) * 0.05)
    ws.add_fem_constant("G", g.MeshFem(mesh, 1, degree=0), np.ones(mesh.nb_convex()))
    ws.add_fixed_size_constant("K", np.array([1.5]))
    ws.add_expression("(-p*Id(3)+2*G*(Sym(Grad_u)-Div_u*Id(3)/3)):Grad_Test_u", mim)
    ws.add_expression("(p+K*Div_u)*Test_p", mim)
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1 + [grp.internal_term(ws)])
    status = L.lib().gfgpu_assemble_host_upper(h, None, None, None)
    assert status == L.E_UNSUPPORTED
