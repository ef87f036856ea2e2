"""Parameter gradients of potentials pinned entry by entry to GWFL's own
symbolic derivative.  The reference fixtures (tests/golden/*_diff.npz, made by
tests/golden/make_golden.py) declare the coefficient as a variable of the
workspace, so the reference's order-1 assembly of the potential holds
dE/du and dE/d(coefficient) (the derivative loop of add_tree,
src/getfem_generic_assembly_workspace.cc:520-535, ga_derivative in
src/getfem_generic_assembly_semantic.cc).  The neo-Hookean energy is written
out in GWFL there (its potential operator has no parameter derivative), and
its energy equals the built-in potential's, which the GPU path lowers.

  kappa*Grad_u.Grad_u      per-element kappa, Q2 and Q4 hexahedra;
                           nodal kappa, Q1 hexahedra (jittered)
  neo-Hookean energy       per-element mu, Q2 hexahedra and P2 tetrahedra
                           (jittered), u = sinusoid modes

GPU: the energy, dE/du and dE/d(coefficient) of getfem_gb300.Potential
(gfgpu_assemble order 0 and 1, gfgpu_potential_gradient) within 1e-12 of
the reference, entry by entry.  CPU: the oracle's energy and dE/du match the
fixtures, and central differences of the oracle's energy agree with the
reference's dE/d(coefficient) (a check of the fixtures themselves)."""
import numpy as np
import pytest

import getfem_gb300 as g

from common import RTOL, load, oracle_problem, slots_of, vec_errors

DIFF_NAMES = ["q2hex_kappa_diff", "q4hex_kappa_diff", "q1hex_kappa_nodal_diff",
              "q2hex_nh_mu_diff", "p2tet_nh_mu_diff"]


def build_diff_case(rec):
    """The GPU-side workspace: the built-in potential, the coefficient as
    per-element (P0) or nodal (S) data."""
    m = rec["meta"]
    kind = "simplex" if m["gt"] == "PK" else "hex"
    mesh = g.Mesh.regular_unit(m["dim"], m["nx"], kind, jitter=rec.get("jitter"))
    mf = g.MeshFem(mesh, m["qdim"], degree=m["degree"])
    mim = g.MeshIm(mesh, m["im"])
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rec["in_u"])
    for cname in m["consts"]:
        ws.add_fixed_size_constant(cname, rec["in_" + cname])
    (vname, vk), = m["vars"].items()
    vmf = g.MeshFem(mesh, 1, degree=0 if vk == "P0" else m["degree"])
    ws.add_fem_constant(vname, vmf, rec["in_" + vname])
    ws.add_expression(m["gpu_expr"], mim)
    return mesh, mf, mim, ws, vname


@pytest.mark.parametrize("name", DIFF_NAMES)
def test_oracle_energy_and_du_match_reference(name):
    rec = load(name)
    mesh, mf, mim, ws, vname = build_diff_case(rec)
    grp = ws.groups[0]
    slots = slots_of(ws)
    E = oracle_problem(mesh, mf, mim, grp.order0, slots).potential(nthreads=1)
    assert abs(E - float(rec["E"][0])) <= RTOL * abs(float(rec["E"][0]))
    dU = oracle_problem(mesh, mf, mim, grp.order1, slots).vector(nthreads=1)
    assert vec_errors(dU, rec["dE_du"]).max() <= RTOL


@pytest.mark.parametrize("name", DIFF_NAMES)
def test_reference_coefficient_gradient_against_oracle_differences(name):
    rec = load(name)
    mesh, mf, mim, ws, vname = build_diff_case(rec)
    grp = ws.groups[0]
    slot = ws.data[vname].slot
    base = slots_of(ws)
    ref = rec["dE_d" + vname]
    rng = np.random.default_rng(9)
    for i in rng.choice(ref.size, 4, replace=False):
        h = 1e-6 * abs(base[slot][i])
        e = []
        for sgn in (1, -1):
            s = dict(base)
            s[slot] = base[slot].copy()
            s[slot][i] += sgn * h
            e.append(oracle_problem(mesh, mf, mim, grp.order0, s).potential(nthreads=1))
        fd = (e[0] - e[1]) / (2 * h)
        assert abs(fd - ref[i]) <= 1e-6 * max(abs(ref[i]), 1e-3 * np.abs(ref).max()), (i, fd, ref[i])


@pytest.mark.gpu
@pytest.mark.parametrize("name", DIFF_NAMES)
def test_gpu_parameter_gradient_matches_gwfl_diff(name):
    torch = pytest.importorskip("torch")
    rec = load(name)
    mesh, mf, mim, ws, vname = build_diff_case(rec)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(rec["in_u"], device=dev, requires_grad=True)
    coef = torch.tensor(rec["in_" + vname], device=dev, requires_grad=True)
    E = pot(u, **{vname: coef})
    E.backward()
    Eref = float(rec["E"][0])
    assert abs(float(E.detach()) - Eref) <= RTOL * abs(Eref)
    assert vec_errors(u.grad.cpu().numpy(), rec["dE_du"]).max() <= RTOL
    assert vec_errors(coef.grad.cpu().numpy(), rec["dE_d" + vname]).max() <= RTOL
