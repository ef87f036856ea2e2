"""Lowering of constant anisotropic gradient couplings to
GFGPU_TERM_GRADGRAD_TENSOR (CPU): the tensor read off the integrand is the
reference's D[(a,k),(b,l)] (test (a,k), trial (b,l)); forms the element
pass cannot assemble symmetrically, potentials and a second anisotropic
source are rejected when the expression is added; the ctypes mirror of
gfgpu_form has the C layout."""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L
from getfem_gb300 import gwfl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
A3 = "[3,0.5,0.25;0.5,2,0.125;0.25,0.125,1]"


def _ws(dim, qdim, degree=1, kind="simplex"):
    mesh = g.Mesh.regular_unit(dim, 2, kind)
    mf = g.MeshFem(mesh, qdim, degree=degree)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    return mesh, mf, ws


def _im(dim):
    return "IM_TRIANGLE(2)" if dim == 2 else "IM_TETRAHEDRON(2)"


def _tensor_terms(terms):
    return [t for t in terms if t["kind"] == L.TERM_GRADGRAD_TENSOR]


def test_matrix_literal_scalar():
    mesh, mf, ws = _ws(3, 1)
    ws.add_expression(f"({A3}*Grad_u).Grad_Test_u + u*Test_u", g.MeshIm(mesh, _im(3)))
    grp = ws.groups[0]
    (t,) = _tensor_terms(grp.order2)
    A = np.array([[3, 0.5, 0.25], [0.5, 2, 0.125], [0.25, 0.125, 1]])
    assert np.array_equal(np.array(t["tensor"]).reshape(3, 3), A)
    assert t["c"][0] is None
    assert [x["kind"] for x in grp.order2 if x is not t] == [L.TERM_MASS]
    assert _tensor_terms(grp.order1) == [t]


def test_per_element_factor_and_isotropic_part():
    mesh, mf, ws = _ws(2, 1, degree=2)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), np.ones(mesh.nb_convex()))
    ws.add_expression("kappa*([2,0.5;0.5,1]*Grad_u).Grad_Test_u + Grad_u.Grad_Test_u",
                      g.MeshIm(mesh, "IM_TRIANGLE(4)"))
    grp = ws.groups[0]
    (t,) = _tensor_terms(grp.order2)
    assert t["c"][0]["kind"] == L.COEF_ELEMENT and t["c"][0]["value"] == 1.0
    assert t["tensor"] == [2.0, 0.5, 0.5, 1.0]
    iso = [x for x in grp.order2 if x["kind"] == L.TERM_GRADGRAD]
    assert len(iso) == 1 and iso[0]["c"][1]["value"] == 1.0


def test_reshaped_stiffness_in_fortran_order():
    rng = np.random.default_rng(4)
    Cst = rng.uniform(-1, 1, (3, 3, 3, 3))
    Cst = Cst + Cst.transpose(2, 3, 0, 1)  # major symmetry
    mesh, mf, ws = _ws(3, 3)
    ws.add_fixed_size_constant("Cani", Cst.ravel(order="F"))
    ws.add_expression("(Reshape(Cani,3,3,3,3):Grad_u):Grad_Test_u", g.MeshIm(mesh, _im(3)))
    (t,) = _tensor_terms(ws.groups[0].order2)
    D = np.array(t["tensor"]).reshape(9, 9)
    for a in range(3):
        for k in range(3):
            for b in range(3):
                for l in range(3):
                    assert D[a * 3 + k, b * 3 + l] == Cst[a, k, b, l]
    form = gwfl.to_form(ws.groups[0].order2)
    assert list(form.tensor)[:81] == list(np.array(t["tensor"]))


@pytest.mark.parametrize("expr,why", [
    ("([1,2;3,4]*Grad_u).Grad_Test_u", "not symmetric"),
    ("([2,0.5;0.5,1]*Grad_u).Grad_u", "potentials"),
    ("kappa*([2,0;0,1]*Grad_u).Grad_Test_u + ([1,0.5;0.5,1]*Grad_u).Grad_Test_u",
     "more than one"),
])
def test_rejected_at_add_time(expr, why):
    mesh, mf, ws = _ws(2, 1)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), np.ones(mesh.nb_convex()))
    with pytest.raises(L.UnsupportedExpression, match=why):
        ws.add_expression(expr, g.MeshIm(mesh, _im(2)))


def test_two_tensor_terms_do_not_share_a_form():
    t = {"kind": L.TERM_GRADGRAD_TENSOR, "scale": 1.0, "field_slot": 0,
         "c": [None, None, None], "tensor": [1.0]}
    with pytest.raises(L.UnsupportedExpression):
        gwfl.to_form([t, dict(t)])


def test_form_layout_matches_the_header():
    if shutil.which("gcc") is None:
        pytest.skip("gcc absent")
    src = ('#include <stdio.h>\n#include <stddef.h>\n#include "gfgpu.h"\n'
           'int main(void) { printf("%zu %zu\\n", sizeof(gfgpu_form), '
           'offsetof(gfgpu_form, tensor)); return 0; }\n')
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(td, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        size, off = map(int, subprocess.run([exe], capture_output=True, text=True,
                                            check=True).stdout.split())
    assert C.sizeof(L.Form) == size
    assert L.Form.tensor.offset == off
