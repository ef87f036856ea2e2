"""GPU parity of the Gauss-point path on hexahedra (GT_QK(3,1), FEM_QK(3,1|2)):
the compressible neo-Hookean tangent and residual, isotropic forms with
constant, per-element and nodal coefficients, mass and load terms, on
jittered (non-affine) meshes.  Pattern bit-exact, K and R within 1e-12
(relative, with a floor of 1e-3 of the row maximum)."""
import numpy as np
import pytest

import getfem_gb300 as g

from common import (RTOL, assert_same_pattern, build_case, golden_csr, load, oracle_problem,
                    slots_of, value_errors, vec_errors)

pytestmark = pytest.mark.gpu

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"


HEX_CASES = ["q2hex_neohookean", "q2hex_neohookean_nodal", "q1hex_nodal_kappa", "q4hex_laplace",
             "q2hex_elastic_nodal"]


@pytest.mark.parametrize("name", HEX_CASES)
def test_gpu_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_case(rec)
    ws.assembly(2)
    K = ws.assembled_matrix()
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    ws.assembly(1)
    assert vec_errors(ws.assembled_vector(), rec["R"]).max() <= RTOL


def hex_case(nx, degree, qdim, im, seed, jitter=True):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.12 * h, 0.12 * h, ((nx + 1) ** 3, 3)) if jitter else None
    mesh = g.Mesh.regular_unit(3, nx, "hex", jitter=jit)
    mf = g.MeshFem(mesh, qdim, degree=degree)
    mim = g.MeshIm(mesh, im)
    return rng, mesh, mf, mim


def check_against_oracle(mesh, mf, mim, ws):
    grp = ws.groups[0]
    slots = slots_of(ws)
    ws.assembly(2)
    K = ws.assembled_matrix()
    Ko = oracle_problem(mesh, mf, mim, grp.order2, slots).matrix(nthreads=4)
    assert_same_pattern(K, Ko)
    ek = value_errors(K, Ko).max()
    ws.assembly(1)
    Ro = oracle_problem(mesh, mf, mim, grp.order1, slots).vector(nthreads=4)
    er = vec_errors(ws.assembled_vector(), Ro).max()
    assert ek <= RTOL and er <= RTOL, (ek, er)


@pytest.mark.parametrize("mu_kind", ["element", "nodal"])
def test_hex_neohookean_jittered(mu_kind):
    rng, mesh, mf, mim = hex_case(3, 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 21)
    xyz = mf.basic_dof_nodes()
    u = 0.04 * np.sin(xyz @ rng.uniform(-3, 3, (3, 3)) + rng.uniform(0, 6, 3)).ravel()
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u)
    if mu_kind == "element":
        ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.3, mesh.nb_convex())))
    else:
        ms = g.MeshFem(mesh, 1, degree=2)
        ws.add_fem_constant("mu", ms, np.exp(rng.normal(0, 0.3, ms.nb_dof())))
    ws.add_fixed_size_constant("D1", np.array([1.5]))
    ws.add_expression(NH, mim)
    check_against_oracle(mesh, mf, mim, ws)


def test_pattern_grows_when_new_entries_appear():
    """At u = 0 the neo-Hookean tangent of an unjittered Q2 mesh has exact
    zeros (F = I: an isotropic tangent with per-element mu); at u != 0 those
    entries are nonzero.  The reference rebuilds K's columns at every
    assembly, so the second assembly must hold them: the gather flags the
    entries missing from the cached pattern and the sync rebuilds it."""
    rng, mesh, mf, mim = hex_case(2, 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 8, jitter=False)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0),
                        np.exp(rng.normal(0, 0.3, mesh.nb_convex())))
    ws.add_fixed_size_constant("D1", np.array([1.5]))
    ws.add_expression(NH, mim)
    ws.assembly(2)
    nnz0 = ws.assembled_matrix().nnz
    xyz = mf.basic_dof_nodes()
    ws.set_variable_value("u", 0.05 * np.sin(xyz @ rng.uniform(-3, 3, (3, 3))).ravel())
    ws.assembly(2)
    K = ws.assembled_matrix()
    Ko = oracle_problem(mesh, mf, mim, ws.groups[0].order2, slots_of(ws)).matrix(nthreads=4)
    assert Ko.nnz > nnz0
    assert_same_pattern(K, Ko)
    assert value_errors(K, Ko).max() <= RTOL


def test_hex_neohookean_q1_reduced():
    rng, mesh, mf, mim = hex_case(4, 1, 3, "IM_GAUSS_PARALLELEPIPED(3,3)", 5)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.02)
    ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0),
                        np.exp(rng.normal(0, 0.3, mesh.nb_convex())))
    ws.add_fixed_size_constant("D1", np.array([0.8]))
    ws.add_expression(NH, mim)
    check_against_oracle(mesh, mf, mim, ws)


ISO = [
    # degree, qdim, im, expression, data
    (1, 1, "IM_GAUSS_PARALLELEPIPED(3,3)",
     "kappa*Grad_u.Grad_Test_u + 3*u*Test_u - f*Test_u", {"kappa": "S", "f": "V"}),
    (2, 1, "IM_GAUSS_PARALLELEPIPED(3,5)",
     "kappa*Grad_u.Grad_Test_u + rho*u*Test_u", {"kappa": "P0", "rho": "S"}),
    (1, 3, "IM_GAUSS_PARALLELEPIPED(3,5)",
     "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "S", "f": "V"}),
    (2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)",
     "lambda*Div_u*Div_Test_u + mu*(Grad_u + Grad_u'):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "P0", "f": "V"}),
]


@pytest.mark.parametrize("case", range(len(ISO)))
def test_hex_isotropic_forms(case):
    degree, qdim, im, expr, data = ISO[case]
    rng, mesh, mf, mim = hex_case(3, degree, qdim, im, 40 + case)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.1)
    for name, kind in data.items():
        if kind == "P0":
            ws.add_fem_constant(name, g.MeshFem(mesh, 1, degree=0),
                                np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        elif kind == "S":
            ms = g.MeshFem(mesh, 1, degree=degree)
            ws.add_fem_constant(name, ms, np.exp(rng.normal(0, 0.2, ms.nb_dof())))
        else:
            ws.add_fem_constant(name, mf, rng.standard_normal(mf.nb_dof()))
    ws.add_expression(expr, mim)
    check_against_oracle(mesh, mf, mim, ws)


def test_hex_deterministic():
    rec = load("q2hex_neohookean")
    mesh, mf, mim, ws = build_case(rec)
    ws.assembly(2)
    K1 = ws.assembled_matrix().copy()
    ws.assembly(2)
    assert np.array_equal(K1.data, ws.assembled_matrix().data)


AFFINE_SF = [
    # degree, im, expression, data: parallelepiped meshes (no jitter), so the
    # vector-only pass is sum-factorised
    (4, "IM_GAUSS_PARALLELEPIPED(3,9)", "kappa*Grad_u.Grad_Test_u", {"kappa": "P0"}),
    (4, "IM_GAUSS_PARALLELEPIPED(3,9)", "kappa*Grad_u.Grad_Test_u + 2*u*Test_u - f*Test_u",
     {"kappa": "P0", "f": "V"}),
    (2, "IM_GAUSS_PARALLELEPIPED(3,5)", "kappa*Grad_u.Grad_Test_u - f*Test_u",
     {"kappa": "P0", "f": "V"}),
    (1, "IM_GAUSS_PARALLELEPIPED(3,3)", "3*Grad_u.Grad_Test_u + u*Test_u", {}),
    (3, "IM_GAUSS_PARALLELEPIPED(3,7)", "kappa*Grad_u.Grad_Test_u", {"kappa": "P0"}),
]


@pytest.mark.parametrize("case", range(len(AFFINE_SF)))
def test_vector_pass_after_pattern(case):
    """A repeated order-1 assembly (pattern built) on parallelepipeds takes the
    vector-only pass: sum-factorised for FEM_QK(3,1|2), whose 1D tables
    reproduce the reference's 3-D basis tables to 1e-14; element tables for
    K >= 3.  Both match the oracle's per-point sums."""
    degree, im, expr, data = AFFINE_SF[case]
    mesh, mf, mim, ws, rng = affine_sf_case(case)
    Ro = oracle_problem(mesh, mf, mim, ws.groups[0].order1, slots_of(ws)).vector(nthreads=4)
    ws.assembly(1)   # first: element matrices formed (the plan's pattern is built)
    e1 = vec_errors(ws.assembled_vector(), Ro).max()
    ws.assembly(1)   # vector only
    e2 = vec_errors(ws.assembled_vector(), Ro).max()
    assert e1 <= RTOL and e2 <= RTOL, (e1, e2)


def affine_sf_case(case):
    degree, im, expr, data = AFFINE_SF[case]
    rng = np.random.default_rng(40 + case)
    nx = 3 if degree <= 2 else 2
    # a sheared but parallelepiped mesh: an affine map of the unit cube
    mesh = g.Mesh.regular_unit(3, nx, "hex")
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, 0.15], [0.05, 0.0, 1.1]])
    mesh.points = np.ascontiguousarray(mesh.points @ A.T)
    mf = g.MeshFem(mesh, 1, degree=degree)
    mim = g.MeshIm(mesh, im)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()))
    for nm, kind in data.items():
        if kind == "P0":
            ws.add_fem_constant(nm, g.MeshFem(mesh, 1, degree=0),
                                np.exp(rng.normal(0, 0.5, mesh.nb_convex())))
        else:
            ws.add_fem_constant(nm, mf, rng.uniform(-1, 1, mf.nb_dof()))
    ws.add_expression(expr, mim)
    return mesh, mf, mim, ws, rng


@pytest.mark.parametrize("case", [0, 1, 4])
def test_opt_in_sum_factorisation_high_order(case):
    """GFGPU_SUM_FACTORISATION on FEM_QK(3,3|4): the exact tensor-product
    basis instead of the reference's monomial evaluation of it (off by up to
    1.5e-10 at K = 4).  R stays within 1e-8 of the reference-exact pass
    (relative, floor 1e-3 of the largest entry) and the call is repeatable
    bit for bit."""
    import ctypes as C
    from getfem_gb300 import _lib as L
    mesh, mf, mim, ws, rng = affine_sf_case(case)
    ws.assembly(1)
    ws.assembly(1)
    Rref = ws.assembled_vector().copy()
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1)
    lib = L.lib()
    out = []
    for _ in range(2):
        L.check(lib.gfgpu_assemble(h, 1, L.SUM_FACTORISATION, None))
        L.check(lib.gfgpu_sync(h))
        v = np.empty(mf.nb_dof())
        L.check(lib.gfgpu_copy_result(h, L.RESULT_VECTOR, v.ctypes.data_as(C.c_void_p)))
        out.append(v)
    assert np.array_equal(out[0], out[1])
    err = vec_errors(out[0], Rref).max()
    assert 0.0 < err <= 1e-8, err


@pytest.mark.parametrize("degree", [1, 3, 4])
def test_vector_pass_axis_aligned(degree):
    """The vector-only pass of kappa*Grad_u.Grad_Test_u on an axis-aligned
    mesh goes through the three diagonal metric tables only (the off-diagonal
    metric terms are exact zeros); it matches the oracle's per-point sums."""
    rng = np.random.default_rng(70 + degree)
    mesh = g.Mesh.regular_unit(3, 2, "hex")
    mf = g.MeshFem(mesh, 1, degree=degree)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,%d)" % (2 * degree + 1))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()))
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0),
                        np.exp(rng.normal(0, 0.5, mesh.nb_convex())))
    ws.add_expression("kappa*Grad_u.Grad_Test_u", mim)
    Ro = oracle_problem(mesh, mf, mim, ws.groups[0].order1, slots_of(ws)).vector(nthreads=4)
    ws.assembly(1)
    ws.assembly(1)   # vector only
    assert vec_errors(ws.assembled_vector(), Ro).max() <= RTOL
