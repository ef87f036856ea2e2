"""Static condensation of an internal im_data variable (the pressure p of a
displacement / pressure pair, one value per element Gauss point), as
ga_workspace::assembly(order, true) does it
(getfem_generic_assembly_compile_and_exec.cc:5562-5790, :8429-8640;
the formulation of tests/test_condensation.cc, on 3-D meshes).

CPU: the oracle against the reference's own outputs (order-1 residual of u
and p, condensed K, condensed vector, internal solution and coupling matrix
KQJpr), and the lowering of the two expressions.  GPU: the same outputs from
the Gauss-point kernel, against the fixtures and against the oracle on
larger meshes; the condensed K of the linear pair equals the elasticity K
with lambda = K - 2 G / 3."""
import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import (RTOL, build_condensed_case, csr_errors, golden_names, load,
                    oracle_problem, vec_errors)

NAMES = golden_names(condensed=True)


def oracle_slots(ws, extra=None):
    slots = {d.slot: np.asarray(d.values, dtype=float) for d in ws.data.values()
             if d.slot >= 0 and d.values is not None}
    slots.update(extra or {})
    return slots


def coupling_csr(rec_or_n, vals, mesh, mf, nq):
    """KQJpr rows (element Gauss points x element DOFs in local order) as a
    CSR of (n + n_int) x n, the internal rows last."""
    import scipy.sparse as sp
    n = mf.nb_dof()
    E, qd = mesh.nb_convex(), mf.qdim
    cols = (mf.dofs[:, :, None] + np.arange(qd)).reshape(E, -1)
    cols = np.repeat(cols, nq, axis=0).ravel()
    rows = n + np.repeat(np.arange(E * nq), cols.size // (E * nq))
    return sp.csr_matrix((np.asarray(vals).ravel(), (rows, cols)), shape=(n + E * nq, n))


def golden_coupling(rec):
    import scipy.sparse as sp
    n, ni = rec["meta"]["n_dof"], rec["meta"]["n_internal"]
    return sp.csr_matrix((rec["C_vals"], rec["C_colidx"], rec["C_rowptr"]), shape=(n + ni, n))


def golden_K(rec):
    import scipy.sparse as sp
    n = rec["meta"]["n_dof"]
    return sp.csr_matrix((rec["K_vals"], rec["K_colidx"], rec["K_rowptr"]), shape=(n, n))


def test_fixtures_present():
    assert set(NAMES) >= {"q2hex_up_condensed", "p2tet_up_condensed_nl"}


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_condensed_case(rec)
    n, nq = mf.nb_dof(), mim.nq
    grp = ws.groups[0]
    ip = grp.internal_term(ws)
    Rf = rec["R_full"]
    slots = oracle_slots(ws, {ip["aux_slot"]: Rf[n:]})
    V, Vint = oracle_problem(mesh, mf, mim, grp.order1 + [ip], slots).vector_internal(nthreads=2)
    assert vec_errors(V, Rf[:n]).max() <= RTOL
    assert vec_errors(Vint, Rf[n:]).max() <= RTOL
    K, Vc, RQ, C = oracle_problem(mesh, mf, mim, grp.order2 + [ip], slots).condensed(nthreads=2)
    assert csr_errors(K, golden_K(rec)).max() <= RTOL
    Rc = rec["Rc"]
    assert vec_errors(Vc, Rc[:n]).max() <= RTOL
    assert vec_errors(RQ, Rc[n:]).max() <= RTOL
    assert csr_errors(coupling_csr(n, C, mesh, mf, nq), golden_coupling(rec)).max() <= RTOL


def test_lowering_of_the_pair():
    rec = load("p2tet_up_condensed_nl")
    mesh, mf, mim, ws = build_condensed_case(rec)
    grp = ws.groups[0]
    ip = grp.internal_term(ws)
    assert ip["kind"] == L.TERM_INTERNAL_P and ip["scale"] == pytest.approx(1.0)
    assert ip["c"][0]["value"] == pytest.approx(-1.0)            # (-p*Id(3)):Grad_Test_u
    assert ip["c"][1]["kind"] == L.COEF_ELEMENT                  # K per element
    assert ip["c"][2]["value"] == pytest.approx(1e3)             # 1e3*pow(p,3)
    gg = [t for t in grp.order2 if t["kind"] == L.TERM_GRADGRAD]
    assert len(gg) == 1
    c = [x["value"] for x in gg[0]["c"]]
    assert c == pytest.approx([1.5 * -2.0 / 3.0, 1.5, 1.5])     # G = 1.5: deviatoric stress


def test_lowering_rejections():
    rec = load("q2hex_up_condensed")
    m = rec["meta"]
    mesh = g.Mesh.regular_unit(3, 1, "hex")
    mf = g.MeshFem(mesh, 3, degree=2)
    mim = g.MeshIm(mesh, m["im"])
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf)
    ws.add_internal_im_variable("p", g.ImData(mim))
    ws.add_fixed_size_constant("K", [2.0])
    for bad in ("Grad_p.Grad_Test_u(1)",                          # im_data: no gradient
                "(p+K*Trace(Grad_u*Grad_u))*Test_p",             # not through Div_u
                "(p+K*Div_u+1)*Test_p",                          # constant term
                "(p*p*Id(3)):Grad_Test_u",                       # not linear in p
                "(p*Grad_u):Grad_Test_u"):                       # p times u
        with pytest.raises(g.UnsupportedExpression):
            ws.add_expression(bad, mim)
    # an internal variable needs both equations, and condensation for order 1
    ws.add_expression("(-p*Id(3)+K*Sym(Grad_u)):Grad_Test_u", mim)
    with pytest.raises(g.UnsupportedExpression):
        ws.groups[0].internal_term(ws)
    ws.add_expression("(p+K*Div_u)*Test_p", mim)
    with pytest.raises(g.GfgpuError):
        ws.assembly(1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_condensation_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_condensed_case(rec)
    n = mf.nb_dof()
    ws.assembly(1, condensation=True)
    V = ws.assembled_vector()
    Rf = rec["R_full"]
    assert V.shape == Rf.shape
    assert vec_errors(V[:n], Rf[:n]).max() <= RTOL
    assert vec_errors(V[n:], Rf[n:]).max() <= RTOL
    # the condensation reads the internal residual from the assembled vector
    ws.assembly(2, condensation=True)
    assert csr_errors(ws.assembled_matrix(), golden_K(rec)).max() <= RTOL
    Vc = ws.assembled_vector()
    Rc = rec["Rc"]
    assert vec_errors(Vc[:n], Rc[:n]).max() <= RTOL
    assert vec_errors(Vc[n:], Rc[n:]).max() <= RTOL
    assert csr_errors(ws.internal_coupling_matrix(), golden_coupling(rec)).max() <= RTOL


def random_pair(kind, nx, degree, im, nonlinear, kb_kind, seed):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, kind, jitter=jit)
    mf = g.MeshFem(mesh, 3, degree=degree)
    mim = g.MeshIm(mesh, im)
    imd = g.ImData(mim)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.05)
    ws.add_internal_im_variable("p", imd, rng.standard_normal(imd.nb_index()) * 0.05)
    E = mesh.nb_convex()
    ws.add_fem_constant("G", g.MeshFem(mesh, 1, degree=0), np.exp(rng.normal(0, 0.2, E)))
    if kb_kind == "nodal":
        ws.add_fem_constant("K", g.MeshFem(mesh, 1, degree=degree),
                            np.exp(rng.normal(0, 0.2, mf.nb_dof() // 3)))
    else:
        ws.add_fixed_size_constant("K", [2.5])
    ws.add_expression("(-p*Id(3)+2*G*(Sym(Grad_u)-Div_u*Id(3)/3)):Grad_Test_u", mim)
    ws.add_expression("((p+1e3*pow(p,3))+K*Div_u)*Test_p" if nonlinear else
                      "(p+K*Div_u)*Test_p", mim)
    return rng, mesh, mf, mim, ws


@pytest.mark.gpu
@pytest.mark.parametrize("case", [("hex", 3, 2, "IM_GAUSS_PARALLELEPIPED(3,5)", True, "nodal"),
                                  ("hex", 4, 1, "IM_GAUSS_PARALLELEPIPED(3,3)", False, "const"),
                                  ("simplex", 3, 2, "IM_TETRAHEDRON(5)", True, "const"),
                                  ("simplex", 3, 1, "IM_TETRAHEDRON(2)", False, "nodal")])
def test_gpu_condensation_matches_oracle(case):
    rng, mesh, mf, mim, ws = random_pair(*case, seed=sum(map(ord, str(case))) % 1000)
    n, nq = mf.nb_dof(), mim.nq
    grp = ws.groups[0]
    ip = grp.internal_term(ws)
    ws.assembly(1, condensation=True)
    V1 = ws.assembled_vector().copy()
    slots = oracle_slots(ws, {ip["aux_slot"]: V1[n:]})
    Vo, Vio = oracle_problem(mesh, mf, mim, grp.order1 + [ip], slots).vector_internal(nthreads=4)
    assert vec_errors(V1[:n], Vo).max() <= RTOL
    assert vec_errors(V1[n:], Vio).max() <= RTOL
    ws.assembly(2, condensation=True)
    K, Vc, RQ, C = oracle_problem(mesh, mf, mim, grp.order2 + [ip], slots).condensed(nthreads=4)
    assert csr_errors(ws.assembled_matrix(), K).max() <= RTOL
    V2 = ws.assembled_vector()
    assert vec_errors(V2[:n], Vc).max() <= RTOL
    assert vec_errors(V2[n:], RQ).max() <= RTOL
    assert csr_errors(ws.internal_coupling_matrix(), coupling_csr(n, C, mesh, mf, nq)).max() <= RTOL


@pytest.mark.gpu
def test_condensed_linear_pair_is_elasticity():
    """With p + K Div_u = 0 eliminated, the deviatoric pair is isotropic
    elasticity with lambda = K - 2 G / 3 and mu = G (assembled here by the
    simplex reference-tensor pass)."""
    rng, mesh, mf, mim, ws = random_pair("simplex", 3, 2, "IM_TETRAHEDRON(5)", False, "const", 7)
    n = mf.nb_dof()
    ws.assembly(1, condensation=True)
    ws.assembly(2, condensation=True)
    Kc = ws.assembled_matrix()
    G = ws.data["G"].values
    ws2 = g.GaWorkspace()
    ws2.add_fem_variable("u", mf)
    mf0 = g.MeshFem(mesh, 1, degree=0)
    ws2.add_fem_constant("lambda", mf0, 2.5 - 2.0 * G / 3.0)
    ws2.add_fem_constant("mu", mf0, G)
    ws2.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u", mim)
    ws2.assembly(2)
    Ke = ws2.assembled_matrix()
    assert abs(Kc - Ke).max() <= 1e-12 * abs(Ke).max()
    assert Kc.shape == (n, n)


@pytest.mark.gpu
def test_condensed_newton_converges():
    """Newton on the nonlinear pair through the condensed system, as the
    model does with internal variables: K' du = -(R_u + Vc), then
    dp = -RQpr - KQJpr du per Gauss point.  The full residual (u rows off
    the clamped face, and every p row) goes to zero quadratically."""
    import scipy.sparse.linalg as spla
    rng, mesh, mf, mim, ws = random_pair("simplex", 3, 2, "IM_TETRAHEDRON(5)", True, "const", 3)
    n = mf.nb_dof()
    ws.clear_expressions()
    f = rng.standard_normal(n)
    ws.add_fem_constant("f", mf, f)
    ws.add_expression("(-p*Id(3)+2*G*(Sym(Grad_u)-Div_u*Id(3)/3)):Grad_Test_u - f.Test_u", mim)
    ws.add_expression("((p+1e3*pow(p,3))+K*Div_u)*Test_p", mim)
    # clamp the DOFs of the nodes on the face x = 0 (DOF 3 k + b: node k, component b)
    free = ~np.repeat(np.abs(mf.basic_dof_nodes()[:, 0]) < 1e-9, 3)
    assert free.sum() < n
    u = np.zeros(n)
    p = np.zeros(ws.nb_internal_dof())
    norms = []
    for it in range(10):
        ws.set_variable_value("u", u)
        ws.set_variable_value("p", p)
        ws.assembly(1, condensation=True)
        R = ws.assembled_vector().copy()
        norms.append(max(np.abs(R[:n][free]).max(), np.abs(R[n:]).max()))
        if norms[-1] <= 1e-13 * norms[0]:
            break
        ws.assembly(2, condensation=True)
        Kc = ws.assembled_matrix().tocsr()
        Vc = ws.assembled_vector()
        KQJ = ws.internal_coupling_matrix().tocsr()[n:]
        du = np.zeros(n)
        du[free] = spla.spsolve(Kc[free][:, free].tocsc(), -(R[:n] + Vc[:n])[free])
        u = u + du
        p = p + (-Vc[n:] - KQJ @ du)
    assert norms[-1] <= 1e-12 * norms[0], norms
    # quadratic convergence in the last steps
    assert len(norms) <= 10 and norms[-2] <= 1e-4 * norms[0], norms
