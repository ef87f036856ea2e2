"""Parity at the full sizes of the benchmark configurations, on the
benchmark's own seeded inputs, against fixtures made by the reference
(tests/golden/make_fullsize.py) and against the oracle run here:

  full_p1tri_poisson_64     64 x 64 P1 triangles (8 192 elements), K and R whole
  full_p2tet_elastic_40     40^3 x 6 P2 tetrahedra (384 000 elements, nnz 133 360 881)
  full_q2hex_neohookean_32  32^3 Q2 hexahedra, neo-Hookean brick form (32 768 elements)
  full_q4hex_laplace_8      8^3 Q4 hexahedra, a sub-mesh of the 64^3 workload

The pattern (nnz, row pointers, column indices) is compared bit for bit
through its SHA-256; values on the fixture's kept rows and entries, R at its
kept positions, and every entry through bilinear probes.  The GPU tests also
compare every entry of K and R with the oracle run on the same host.

The CPU tests pin the oracle itself at these sizes (same hashes and values
as the reference)."""
import os

import numpy as np
import pytest

import bench
import getfem_gb300 as g

from common import (RTOL, assert_fullsize, assert_same_pattern, fullsize_report, load,
                    oracle_problem, slots_of, vec_errors)

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"


def build_full(name, inputs=None):
    """Mesh, MeshFem, MeshIm and GaWorkspace of a full-size case with the
    benchmark's inputs (the generators of bench.py); `inputs`, when given,
    receives the generated arrays under the fixture's names."""
    inputs = {} if inputs is None else inputs
    if name == "full_p1tri_poisson_64":
        mesh = g.Mesh.regular_unit(2, 64, "simplex")
        mf = g.MeshFem(mesh, 1, degree=1)
        mim = g.MeshIm(mesh, "IM_TRIANGLE(2)")
        inputs.update(u=np.zeros(mf.nb_dof()), f=bench.poisson_inputs(mf.nb_dof()))
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=inputs["u"])
        ws.add_fem_constant("f", mf, inputs["f"])
        ws.add_expression("Grad_u.Grad_Test_u - f*Test_u", mim)
        return mesh, mf, mim, ws
    if name == "full_p2tet_elastic_40":
        mesh, mf, mim, ws, d = bench.make_problem(40)
        jit, _ = bench.p2tet_inputs(40)
        inputs.update(u=d["u"], **{"lambda": d["lam"]}, mu=d["mu"], f=d["f"], jitter=jit)
        return mesh, mf, mim, ws
    if name == "full_q2hex_neohookean_32":
        mesh = g.Mesh.regular_unit(3, 32, "hex")
        mf = g.MeshFem(mesh, 3, degree=2)
        mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
        u, mu = bench.neohookean_inputs(mf.basic_dof_nodes(), mesh.nb_convex())
        inputs.update(u=u, mu=mu, D1=np.array([1.5]))
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=u)
        ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0), mu)
        ws.add_fixed_size_constant("D1", np.array([1.5]))
        ws.add_expression(NH, mim)
        return mesh, mf, mim, ws
    if name == "full_q4hex_laplace_8":
        mesh = g.Mesh.regular_unit(3, 8, "hex")
        mf = g.MeshFem(mesh, 1, degree=4)
        mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,9)")
        kappa, u = bench.q4_inputs(mesh.nb_convex(), mf.nb_dof())
        inputs.update(u=u, kappa=kappa)
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=u)
        ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), kappa)
        ws.add_expression("kappa*Grad_u.Grad_Test_u", mim)
        return mesh, mf, mim, ws
    raise KeyError(name)


def assert_same_inputs(rec, inputs):
    """The generated inputs are those the reference assembled (same bits)."""
    import hashlib
    for k, h in rec["meta"]["input_sha256"].items():
        got = hashlib.sha256(np.ascontiguousarray(inputs[k], dtype="<f8").tobytes()).hexdigest()
        assert got == h, f"input {k} differs from the fixture's (the generator gave other bits)"


NAMES = ["full_p1tri_poisson_64", "full_q4hex_laplace_8", "full_q2hex_neohookean_32",
         "full_p2tet_elastic_40"]


def _oracle(mesh, mf, mim, ws, nthreads):
    grp = ws.groups[0]
    slots = slots_of(ws)
    K = oracle_problem(mesh, mf, mim, grp.order2, slots).matrix(nthreads=nthreads)
    R = oracle_problem(mesh, mf, mim, grp.order1, slots).vector(nthreads=nthreads)
    return K, R


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_at_full_size(name):
    """The oracle is pinned at the configurations' sizes too."""
    rec = load(name)
    inputs = {}
    mesh, mf, mim, ws = build_full(name, inputs)
    assert_same_inputs(rec, inputs)
    assert mf.nb_dof() == rec["meta"]["n_dof"]
    K, R = _oracle(mesh, mf, mim, ws, os.cpu_count() or 1)
    assert_fullsize(fullsize_report(rec, K.indptr, K.indices, K.data, R))


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_reference_and_oracle_at_full_size(name):
    rec = load(name)
    inputs = {}
    mesh, mf, mim, ws = build_full(name, inputs)
    assert_same_inputs(rec, inputs)
    ws.assembly(2)
    K = ws.assembled_matrix()
    ws.assembly(1)
    R = np.asarray(ws.assembled_vector())
    assert_fullsize(fullsize_report(rec, K.indptr, K.indices, K.data, R))
    # every entry against the oracle run on this host
    Ko, Ro = _oracle(mesh, mf, mim, ws, os.cpu_count() or 1)
    assert_same_pattern(K, Ko)
    d = np.abs(np.asarray(K.data) - Ko.data)
    rows = np.repeat(np.arange(Ko.shape[0]), np.diff(Ko.indptr))
    from common import _row_max, FLOOR
    rmax = _row_max(np.asarray(Ko.indptr, dtype=np.int64), Ko.data)
    scale = np.maximum(np.abs(Ko.data), FLOOR * rmax[rows])
    scale[scale == 0] = 1.0
    assert float((d / scale).max()) <= RTOL
    assert float(vec_errors(R, Ro).max()) <= RTOL
