"""The autotuner (gfgpu_tune): threads per element of the element pass and
warps per block of the row gather, per element family.

Every launch configuration computes each entry with the same operations in
the same order, so K and R must be the same bits for every candidate and for
the tuned choice, on the three element-kernel families (affine simplices,
Gauss-point hexahedra with the neo-Hookean law, parallelepiped hexahedra).
The recorded configurations are written to and read back from a file, and a
plan created afterwards starts with them.  The file format is also checked
on the CPU."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"


def _case(name):
    rng = np.random.default_rng(17)
    if name == "p2tet_elastic":
        nx = 4
        h = 1.0 / nx
        jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
        mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
        mf = g.MeshFem(mesh, 3, degree=2)
        mf0 = g.MeshFem(mesh, 1, degree=0)
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 1e-3)
        ws.add_fem_constant("lambda", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        ws.add_fem_constant("mu", mf0, np.exp(rng.normal(0, 0.2, mesh.nb_convex())))
        ws.add_fem_constant("f", mf, rng.standard_normal(mf.nb_dof()))
        ws.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
                          g.MeshIm(mesh, "IM_TETRAHEDRON(5)"))
    elif name == "q2hex_neohookean":
        mesh = g.Mesh.regular_unit(3, 3, "hex")
        mf = g.MeshFem(mesh, 3, degree=2)
        xyz = mf.basic_dof_nodes()
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=(0.05 * np.sin(xyz @ rng.uniform(-3, 3, (3, 3)))).ravel())
        ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.3, mesh.nb_convex())))
        ws.add_fixed_size_constant("D1", np.array([1.5]))
        ws.add_expression(NH, g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)"))
    elif name == "q4hex_laplace":
        mesh = g.Mesh.regular_unit(3, 3, "hex")
        mf = g.MeshFem(mesh, 1, degree=4)
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()))
        ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0),
                            np.exp(rng.normal(0, 0.5, mesh.nb_convex())))
        ws.add_expression("kappa*Grad_u.Grad_Test_u", g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,9)"))
    else:
        raise KeyError(name)
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1)
    ws._upload(h, grp.order1, need_u=True)
    return ws, mf, h


def _assemble(h, n):
    lib = L.lib()
    L.check(lib.gfgpu_assemble(h, 2, L.WITH_VECTOR, None))
    L.check(lib.gfgpu_sync(h))
    nr, nnz = C.c_int64(), C.c_int64()
    L.check(lib.gfgpu_pattern_size(h, C.byref(nr), C.byref(nnz)))
    vals = np.empty(nnz.value)
    vec = np.empty(n)
    L.check(lib.gfgpu_copy_result(h, L.RESULT_VALUES, vals.ctypes.data))
    L.check(lib.gfgpu_copy_result(h, L.RESULT_VECTOR, vec.ctypes.data))
    return vals, vec


def _launch(h):
    l = L.Launch()
    L.check(L.lib().gfgpu_get_launch(h, C.byref(l)))
    return l.ep_threads, l.gather_warps


@pytest.mark.gpu
@pytest.mark.parametrize("name,eps", [("p2tet_elastic", (2, 4, 8)),
                                      ("q2hex_neohookean", (128, 256, 512)),
                                      ("q4hex_laplace", (128, 256, 512))])
def test_every_launch_configuration_gives_the_same_bits(name, eps):
    ws, mf, h = _case(name)
    lib = L.lib()
    default = _launch(h)
    K0, R0 = _assemble(h, mf.nb_dof())
    for ep in eps:
        for gw in (2, 4, 8):
            l = L.Launch(ep, gw)
            L.check(lib.gfgpu_set_launch(h, C.byref(l)))
            K, R = _assemble(h, mf.nb_dof())
            assert np.array_equal(K, K0) and np.array_equal(R, R0), (ep, gw)
    bad = L.Launch(3, 4)
    assert lib.gfgpu_set_launch(h, C.byref(bad)) == L.E_INVALID
    best = L.Launch()
    L.check(lib.gfgpu_tune(h, 2, C.byref(best)))
    assert best.ep_threads in eps and best.gather_warps in (2, 4, 8)
    assert _launch(h) == (best.ep_threads, best.gather_warps)
    K, R = _assemble(h, mf.nb_dof())
    assert np.array_equal(K, K0) and np.array_equal(R, R0)
    assert default[0] in eps


@pytest.mark.gpu
def test_recorded_configuration_is_saved_loaded_and_used_by_new_plans():
    lib = L.lib()
    ws, mf, h = _case("p2tet_elastic")
    L.check(lib.gfgpu_set_launch(h, C.byref(L.Launch(8, 2))))
    best = L.Launch()
    L.check(lib.gfgpu_tune(h, 1, C.byref(best)))
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "tuned.txt").encode()
        L.check(lib.gfgpu_tune_save(path))
        lines = open(path).read().splitlines()
        mine = [ln for ln in lines if ln.startswith("simplex-d3-")]
        assert mine and mine[0].split()[1:] == [str(best.ep_threads), str(best.gather_warps)]
        # a different recorded configuration, loaded, is what a new plan starts with
        other = 2 if best.ep_threads != 2 else 8
        with open(path, "w") as f:
            f.write(f"{mine[0].split()[0]} {other} 8\n")
        L.check(lib.gfgpu_tune_load(path))
    ws2, mf2, h2 = _case("p2tet_elastic")
    assert _launch(h2) == (other, 8)


def test_tune_file_format_is_checked():
    lib = L.lib()
    with tempfile.TemporaryDirectory() as td:
        good = os.path.join(td, "good.txt")
        with open(good, "w") as f:
            f.write("simplex-d3-k0-p2-q3-nq15-law0|some_gpu 4 2\n"
                    "gauss-d3-k1-p2-q3-nq27-law1|some_gpu 128 8\n")
        assert lib.gfgpu_tune_load(good.encode()) == L.OK
        out = os.path.join(td, "out.txt")
        assert lib.gfgpu_tune_save(out.encode()) == L.OK
        text = open(out).read()
        assert "simplex-d3-k0-p2-q3-nq15-law0|some_gpu 4 2" in text
        assert "gauss-d3-k1-p2-q3-nq27-law1|some_gpu 128 8" in text
        bad = os.path.join(td, "bad.txt")
        with open(bad, "w") as f:
            f.write("simplex-d3-k0-p2-q3-nq15-law0|some_gpu 5 2\n")
        assert lib.gfgpu_tune_load(bad.encode()) == L.E_INVALID
        with open(bad, "w") as f:
            f.write("simplex-d3 4\n")
        assert lib.gfgpu_tune_load(bad.encode()) == L.E_INVALID
        assert lib.gfgpu_tune_load(os.path.join(td, "missing.txt").encode()) == L.E_INVALID
