"""GPU parity of the affine-simplex path against the reference fixtures and
the oracle: sparsity pattern bit-exact, K and R within 1e-12 (relative, with
a floor of 1e-3 of the row maximum), results reproducible bit for bit."""
import ctypes as C

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import (RTOL, assert_same_pattern, build_case, golden_csr, load, oracle_problem,
                    slots_of, value_errors, vec_errors)

pytestmark = pytest.mark.gpu

SIMPLEX_CASES = ["p1tri_poisson", "p2tri_poisson_kappa", "p1tri_mass_laplace", "p2tri_elastic",
                 "p1tet_elastic", "p2tet_elastic", "p2tet_elastic_alt", "p2tet_poisson"]


@pytest.mark.parametrize("name", SIMPLEX_CASES)
def test_gpu_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_case(rec)
    ws.assembly(2)
    K = ws.assembled_matrix()
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    ws.assembly(1)
    R = ws.assembled_vector()
    assert vec_errors(R, rec["R"]).max() <= RTOL


def elastic_problem(nx, seed=3, degree=2):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
    mf = g.MeshFem(mesh, 3, degree=degree)
    mf0 = g.MeshFem(mesh, 1, degree=0)
    mim = g.MeshIm(mesh, "IM_TETRAHEDRON(5)" if degree == 2 else "IM_TETRAHEDRON(2)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.01)
    ws.add_fem_constant("lambda", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
    ws.add_fem_constant("mu", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
    ws.add_fem_constant("f", mf, rng.standard_normal(mf.nb_dof()))
    ws.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u", mim)
    return mesh, mf, mim, ws


def test_gpu_matches_oracle_larger():
    mesh, mf, mim, ws = elastic_problem(6)
    ws.assembly(2)
    K = ws.assembled_matrix()
    grp = ws.groups[0]
    Ko = oracle_problem(mesh, mf, mim, grp.order2, slots_of(ws)).matrix(nthreads=4)
    assert_same_pattern(K, Ko)
    assert value_errors(K, Ko).max() <= RTOL
    ws.assembly(1)
    Ro = oracle_problem(mesh, mf, mim, grp.order1, slots_of(ws)).vector(nthreads=4)
    assert vec_errors(ws.assembled_vector(), Ro).max() <= RTOL


def test_gpu_deterministic_and_fused_pass():
    mesh, mf, mim, ws = elastic_problem(5, seed=11)
    ws.assembly(2)
    K1 = ws.assembled_matrix().copy()
    ws.assembly(2)
    K2 = ws.assembled_matrix()
    assert np.array_equal(K1.data, K2.data)  # no atomics: bit-identical
    ws.assembly(1)
    R1 = ws.assembled_vector().copy()
    # K and R in one pass through the C ABI with host buffers
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1)
    u = np.ascontiguousarray(ws.data["u"].values)
    nr, nnz = C.c_int64(), C.c_int64()
    lib = L.lib()
    L.check(lib.gfgpu_assemble(h, 2, 0, None))
    L.check(lib.gfgpu_pattern_size(h, C.byref(nr), C.byref(nnz)))
    vals = np.empty(nnz.value)
    vec = np.empty(nr.value)
    L.check(lib.gfgpu_assemble_host(h, u.ctypes.data_as(C.c_void_p),
                                    vals.ctypes.data_as(C.c_void_p), vec.ctypes.data_as(C.c_void_p)))
    # the fused pass forms R as (row . u) + dropped contributions: the same
    # sum in another order, equal within the tolerance
    assert vec_errors(vec, R1).max() <= RTOL
    assert np.array_equal(vals, K1.data)
    vec2 = np.empty(nr.value)
    L.check(lib.gfgpu_assemble_host(h, u.ctypes.data_as(C.c_void_p), None,
                                    vec2.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(vec, vec2)
    # page-locked host buffers: the gather writes them directly
    torch = pytest.importorskip("torch")
    pv = torch.empty(nnz.value, dtype=torch.float64).pin_memory()
    pr = torch.empty(nr.value, dtype=torch.float64).pin_memory()
    L.check(lib.gfgpu_assemble_host(h, u.ctypes.data_as(C.c_void_p), C.c_void_p(pv.data_ptr()),
                                    C.c_void_p(pr.data_ptr())))
    assert np.array_equal(pv.numpy(), vals) and np.array_equal(pr.numpy(), vec)


def test_degenerate_element_reports_jacobian_error():
    mesh = g.Mesh.regular_unit(2, 3, "simplex")
    cv = mesh.cvpts.copy()
    cv[4, 1] = cv[4, 0]  # a flat triangle: det K = 0
    bad = g.Mesh(2, L.SIMPLEX, mesh.points, cv)
    mf = g.MeshFem(bad, 1, degree=1)
    mim = g.MeshIm(bad, "IM_TRIANGLE(2)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf)
    ws.add_expression("Grad_u.Grad_Test_u", mim)
    with pytest.raises(g.GfgpuError) as ei:
        ws.assembly(2)
    assert ei.value.status == L.E_JACOBIAN


def test_unsupported_expressions_rejected_at_add_time():
    mesh = g.Mesh.regular_unit(2, 2, "simplex")
    mf = g.MeshFem(mesh, 1, degree=1)
    mim = g.MeshIm(mesh, "IM_TRIANGLE(2)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf)
    for expr in ["Grad_u.Grad_u*Grad_u.Grad_Test_u", "u*Grad_u(1)*Test_u", "Hess_u(1,1)*Test_u",
                 "[1;2].Grad_Test_u*u"]:
        with pytest.raises(g.UnsupportedExpression):
            ws.add_expression(expr, mim)
