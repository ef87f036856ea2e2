"""Constant anisotropic gradient couplings (GFGPU_TERM_GRADGRAD_TENSOR) on
affine simplices.  GPU parity with the reference fixtures:
  * a symmetric matrix literal times a per-element coefficient, plus an
    isotropic Laplacian and a load, on P2 triangles;
  * a matrix literal with a mass term on P1 tetrahedra;
  * a Reshape'd 4th-order stiffness (major and minor symmetry) on P2
    tetrahedra.
Also against the oracle on a larger jittered mesh, reproducible bit for bit;
the paths that do not lower the term (hexahedra, batches) refuse it with a
status instead of assembling something else.
Sparsity pattern bit-exact; K and R within 1e-12 (relative, with a floor of
1e-3 of the row maximum)."""
import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import (RTOL, assert_same_pattern, build_case, golden_csr, load, oracle_problem,
                    slots_of, value_errors, vec_errors)

pytestmark = pytest.mark.gpu

ANISO_CASES = ["p2tri_aniso_kappa", "p1tet_aniso_mass", "p2tet_aniso_elastic"]


@pytest.mark.parametrize("name", ANISO_CASES)
def test_gpu_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_case(rec)
    assert any(t["kind"] == L.TERM_GRADGRAD_TENSOR for t in ws.groups[0].order2)
    ws.assembly(2)
    K = ws.assembled_matrix()
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    ws.assembly(1)
    R = ws.assembled_vector()
    assert vec_errors(R, rec["R"]).max() <= RTOL


def stiffness(rng):
    """C[a,k,b,l] = S[V(a,k), V(b,l)], S a random symmetric positive definite
    Voigt matrix: major and minor symmetry exactly."""
    M = rng.uniform(-0.3, 0.3, (6, 6))
    S = (M + M.T) / 2 + np.diag(rng.uniform(1.0, 3.0, 6))
    V = [[0, 5, 4], [5, 1, 3], [4, 3, 2]]
    C = np.zeros((3, 3, 3, 3))
    for a in range(3):
        for k in range(3):
            for b in range(3):
                for l in range(3):
                    C[a, k, b, l] = S[V[a][k], V[b][l]]
    return C


def aniso_elastic_problem(nx, seed=11):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
    mf = g.MeshFem(mesh, 3, degree=2)
    mf0 = g.MeshFem(mesh, 1, degree=0)
    mim = g.MeshIm(mesh, "IM_TETRAHEDRON(5)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.01)
    ws.add_fixed_size_constant("Cani", stiffness(rng).ravel(order="F"))
    ws.add_fem_constant("theta", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
    ws.add_fem_constant("f", mf, rng.standard_normal(mf.nb_dof()))
    ws.add_expression("theta*(Reshape(Cani,3,3,3,3):Grad_u):Grad_Test_u - f.Test_u", mim)
    return mesh, mf, mim, ws


def test_aniso_elastic_matches_oracle_larger_and_is_reproducible():
    mesh, mf, mim, ws = aniso_elastic_problem(6)
    grp = ws.groups[0]
    ws.assembly(2)
    K = ws.assembled_matrix().copy()
    Ko = oracle_problem(mesh, mf, mim, grp.order2, slots_of(ws)).matrix(nthreads=4)
    assert_same_pattern(K, Ko)
    assert value_errors(K, Ko).max() <= RTOL
    # K is symmetric bit for bit (the upper node blocks are stored)
    assert (K != K.T).nnz == 0
    ws.assembly(2)
    assert np.array_equal(ws.assembled_matrix().data, K.data)
    ws.assembly(1)
    R = ws.assembled_vector().copy()
    Ro = oracle_problem(mesh, mf, mim, grp.order1, slots_of(ws)).vector(nthreads=4)
    assert vec_errors(R, Ro).max() <= RTOL


def test_batch_refuses_anisotropic_plans():
    from getfem_gb300.batch import Batch
    ws = aniso_elastic_problem(2, seed=21)[3]
    ws.assembly(2)
    with pytest.raises(L.GfgpuError):
        Batch([ws])


def test_hexahedra_refuse_the_tensor_coupling():
    mesh = g.Mesh.regular_unit(3, 2, "hex")
    mf = g.MeshFem(mesh, 1, degree=1)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,3)")
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    with pytest.raises(L.GfgpuError):
        ws.add_expression("([3,0.5,0.25;0.5,2,0.125;0.25,0.125,1]*Grad_u).Grad_Test_u", mim)
        ws.assembly(2)
