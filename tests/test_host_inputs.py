"""Host-side inputs of the hot path against the reference's own outputs:
regular_unit_mesh points and convexes, mesh_fem DOF numbering, integration
points and weights, base values and gradients."""
import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import build_case, golden_names, load


@pytest.mark.parametrize("name", golden_names())
def test_mesh_and_dofs_match_reference(name):
    rec = load(name)
    mesh, mf, mim, _ = build_case(rec)
    # coordinates are computed as the reference computes them: bit-identical
    assert np.array_equal(mesh.points, rec["points"])
    assert np.array_equal(mesh.cvpts, rec["cvpts"])
    assert np.array_equal(mf.dofs, rec["dofs"])
    assert mf.nb_dof() == rec["meta"]["n_dof"]
    mf0 = g.MeshFem(mesh, 1, degree=0)
    assert np.array_equal(mf0.dofs.ravel(), rec["dofs0"])


@pytest.mark.parametrize("name", golden_names())
def test_tables_match_reference(name):
    rec = load(name)
    m = rec["meta"]
    mesh, mf, mim, _ = build_case(rec)
    pts, w = mim.points_weights()
    np.testing.assert_allclose(pts, rec["im_points"], rtol=0, atol=2e-15)
    np.testing.assert_allclose(w, rec["im_weights"], rtol=2e-15, atol=0)
    import ctypes as C
    nq, nb, dim = pts.shape[0], mf.nb, m["dim"]
    val = np.empty((nq, nb))
    grad = np.empty((nq, nb, dim))
    L.check(L.lib().gfgpu_basis_tables(dim, mesh.kind, mf.degree, mim.im.encode(),
                                       val.ctypes.data_as(C.c_void_p),
                                       grad.ctypes.data_as(C.c_void_p)))
    ref_val = rec["base_val"].reshape(nq, nb)
    # base_tensor of grad_base_value is (nb, 1, dim), first index fastest
    ref_grad = rec["base_grad"].reshape(nq, dim, nb).transpose(0, 2, 1)
    np.testing.assert_allclose(val, ref_val, rtol=0, atol=1e-13)
    np.testing.assert_allclose(grad, ref_grad, rtol=0, atol=1e-12)


def test_unit_mesh_sizes():
    m = g.Mesh.regular_unit(3, 4, "simplex")
    assert m.nb_convex() == 6 * 64 and m.nb_points() == 125
    m = g.Mesh.regular_unit(3, 4, "hex")
    assert m.nb_convex() == 64 and m.nb_points() == 125
    mf = g.MeshFem(m, 3, degree=2)
    assert mf.nb_dof() == 3 * 9 ** 3


def test_bad_inputs_raise():
    with pytest.raises(g.GfgpuError):
        g.Mesh.regular_unit(4, 2)
    with pytest.raises(g.UnsupportedExpression):
        g.MeshIm(g.Mesh.regular_unit(2, 2), "IM_NOT_A_METHOD(3)")
