"""Generates the golden fixtures under tests/golden/ from the reference GetFEM
build (oracle/_ref/ref_driver, made by `make -C oracle/refbuild`).

Each case builds a structured unit mesh with getfem::regular_unit_mesh,
feeds seeded input vectors to the reference's own ga_workspace
(add_expression + assembly), and stores inputs and outputs: mesh points and
convexes, DOF maps, integration points and weights, base values and
gradients, the assembled K as CSR (rows = test DOFs) and R.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"
NH_POT = "Compressible_Neo_Hookean_potential(Grad_u,[0.5*mu;D1])"

# name, dim, gt, degree, qdim, im, nx, expr, consts{name: kind}, jitter, u kind
CASES = [
    ("p1tri_poisson", 2, "PK", 1, 1, "IM_TRIANGLE(2)", 8,
     "Grad_u.Grad_Test_u - f*Test_u", {"f": "V"}, False, "normal"),
    ("p2tri_poisson_kappa", 2, "PK", 2, 1, "IM_TRIANGLE(4)", 5,
     "kappa*Grad_u.Grad_Test_u - f*Test_u", {"kappa": "P0", "f": "V"}, True, "normal"),
    ("p1tri_mass_laplace", 2, "PK", 1, 1, "IM_TRIANGLE(2)", 6,
     "2*u*Test_u + Grad_u.Grad_Test_u", {}, False, "normal"),
    ("p2tri_elastic", 2, "PK", 2, 2, "IM_TRIANGLE(4)", 4,
     "(lambda*Div_u*Id(2)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "P0", "f": "V"}, True, "normal"),
    ("p1tet_elastic", 3, "PK", 1, 3, "IM_TETRAHEDRON(2)", 3,
     "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "P0", "f": "V"}, True, "normal"),
    ("p2tet_elastic", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 3,
     "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "P0", "f": "V"}, True, "normal"),
    ("p2tet_elastic_alt", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 3,
     "lambda*Div_u*Div_Test_u + mu*(Grad_u + Grad_u'):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "P0", "f": "V"}, True, "normal"),
    ("p2tet_poisson", 3, "PK", 2, 1, "IM_TETRAHEDRON(5)", 3,
     "Grad_u.Grad_Test_u", {}, True, "normal"),
    ("q2hex_neohookean", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 2,
     NH, {"mu": "P0", "D1": "C"}, False, "modes"),
    ("q4hex_laplace", 3, "QK", 4, 1, "IM_GAUSS_PARALLELEPIPED(3,9)", 2,
     "kappa*Grad_u.Grad_Test_u", {"kappa": "P0"}, False, "normal"),
    ("q1hex_nodal_kappa", 3, "QK", 1, 1, "IM_GAUSS_PARALLELEPIPED(3,3)", 3,
     "kappa*Grad_u.Grad_Test_u + 3*u*Test_u - f*Test_u", {"kappa": "S", "f": "V"}, True,
     "normal"),
    ("q2hex_elastic_nodal", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 2,
     "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u",
     {"lambda": "P0", "mu": "S", "f": "V"}, True, "normal"),
    ("q2hex_neohookean_nodal", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 3,
     NH, {"mu": "S", "D1": "C"}, True, "modes"),
    # potentials: order 0 is the energy, orders 1 and 2 the reference's
    # symbolic derivatives of it (GWFL Diff)
    ("q2hex_nh_potential", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 3,
     NH_POT, {"mu": "P0", "D1": "C"}, True, "modes"),
    ("p2tet_nh_potential", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 2,
     NH_POT, {"mu": "P0", "D1": "C"}, True, "modes"),
    ("q2hex_kappa_potential", 3, "QK", 2, 1, "IM_GAUSS_PARALLELEPIPED(3,5)", 3,
     "kappa*Grad_u.Grad_u", {"kappa": "P0"}, False, "normal"),
    ("p2tri_energy_potential", 2, "PK", 2, 1, "IM_TRIANGLE(4)", 5,
     "kappa*Grad_u.Grad_u + 2*u*u - f*u", {"kappa": "P0", "f": "V"}, True, "normal"),
]
# Poisson on the 64 x 64 P1 triangle mesh, homogeneous Dirichlet conditions
# on the boundary, solved by gmm::cg (the 2-D Poisson configuration)
CASES.append(("p1tri_poisson_cg", 2, "PK", 1, 1, "IM_TRIANGLE(2)", 64,
              "Grad_u.Grad_Test_u - f*Test_u", {"f": "V"}, False, "zero"))
EXTRA = {"p1tri_poisson_cg": ["solve=cg", "resmax=1e-12", "maxiter=100000"]}
# Constant anisotropic gradient couplings: a symmetric matrix literal for
# scalar fields, and a 4th-order stiffness with major and minor symmetry
# (a fixed-size constant of 81 values, Reshape'd in the expression) for 3-D
# elasticity
CASES += [
    ("p2tri_aniso_kappa", 2, "PK", 2, 1, "IM_TRIANGLE(4)", 5,
     "kappa*([2,0.5;0.5,1]*Grad_u).Grad_Test_u + Grad_u.Grad_Test_u - f*Test_u",
     {"kappa": "P0", "f": "V"}, True, "normal"),
    ("p1tet_aniso_mass", 3, "PK", 1, 1, "IM_TETRAHEDRON(2)", 4,
     "([3,0.5,0.25;0.5,2,0.125;0.25,0.125,1]*Grad_u).Grad_Test_u + u*Test_u",
     {}, True, "normal"),
    ("p2tet_aniso_elastic", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 3,
     "(Reshape(Cani,3,3,3,3):Grad_u):Grad_Test_u - f.Test_u",
     {"Cani": "C", "f": "V"}, True, "normal"),
    # the same couplings on jittered (non-affine) hexahedra: they pin the
    # oracle's per-point contraction for the hexahedral kernels
    ("q2hex_aniso", 3, "QK", 2, 1, "IM_GAUSS_PARALLELEPIPED(3,5)", 2,
     "([3,0.5,0.25;0.5,2,0.125;0.25,0.125,1]*Grad_u).Grad_Test_u - f*Test_u",
     {"f": "V"}, True, "normal"),
    ("q1hex_aniso_elastic", 3, "QK", 1, 3, "IM_GAUSS_PARALLELEPIPED(3,3)", 2,
     "(Reshape(Cani,3,3,3,3):Grad_u):Grad_Test_u", {"Cani": "C"}, True, "normal"),
]


def stiffness_tensor(rng) -> np.ndarray:
    """C[a,k,b,l] = S[V(a,k), V(b,l)] for a random symmetric positive
    definite 6 x 6 (Voigt) matrix S: major and minor symmetry exactly."""
    M = rng.uniform(-0.3, 0.3, (6, 6))
    S = (M + M.T) / 2 + np.diag(rng.uniform(1.0, 3.0, 6))
    voigt = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (1, 2): 3, (2, 1): 3, (0, 2): 4, (2, 0): 4,
             (0, 1): 5, (1, 0): 5}
    C = np.zeros((3, 3, 3, 3))
    for a in range(3):
        for k in range(3):
            for b in range(3):
                for l in range(3):
                    C[a, k, b, l] = S[voigt[a, k], voigt[b, l]]
    return C
# Mixed displacement / pressure forms with the pressure p an internal im_data
# variable (one value per element Gauss point), condensed at order 2: the
# formulation of the reference's condensation test (tests/test_condensation.cc,
# DIFFICULTY 0 and 1) on 3-D meshes.
UP_A = "(-p*Id(3)+2*G*(Sym(Grad_u)-Div_u*Id(3)/3)):Grad_Test_u"
# name, dim, gt, degree, qdim, im, nx, u-equation, p-equation, consts, jitter
CONDENSE_CASES = [
    ("q2hex_up_condensed", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 2,
     UP_A, "(p+K*Div_u)*Test_p", {"G": "P0", "K": "C"}, True),
    ("p2tet_up_condensed_nl", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 2,
     UP_A, "((p+1e3*pow(p,3))+K*Div_u)*Test_p", {"G": "C", "K": "P0"}, True),
]
ORDERS = {"q2hex_nh_potential": "0,1,2", "p2tet_nh_potential": "0,1,2",
          "q2hex_kappa_potential": "0,1,2", "p2tri_energy_potential": "0,1,2"}


# Parameter gradients of potentials from GWFL's own symbolic derivative: the
# coefficient is declared as a variable (ref_driver vars=...), so the
# reference's order-1 assembly of the potential holds dE/du and dE/dcoef.
# The neo-Hookean energy is written out in GWFL (the law's potential
# operator has no parameter derivative, getfem_nonlinear_elasticity.cc:1812):
# W = C1 (j1 - 3) + D1 (sqrt(i3) - 1)^2, C = F'F, j1 = tr(C) det(C)^(-1/3)
# (the law's strain_energy, getfem_nonlinear_elasticity.cc:503-523), with
# C1 = mu/2; `gpu_expr` is the built-in potential the GPU path lowers, whose
# energy must equal the explicit one.
_F = "(Id(3)+Grad_u)"
NH_EXPLICIT = (f"0.5*mu*(Trace({_F}'*{_F})*pow(Det({_F}'*{_F}),-1/3) - 3)"
               f" + D1*sqr(sqrt(Det({_F}'*{_F})) - 1)")
# name, dim, gt, degree, qdim, im, nx, expr, gpu_expr, consts, vars, jitter, u kind
DIFF_CASES = [
    ("q2hex_kappa_diff", 3, "QK", 2, 1, "IM_GAUSS_PARALLELEPIPED(3,5)", 3,
     "kappa*Grad_u.Grad_u", "kappa*Grad_u.Grad_u", {}, {"kappa": "P0"}, False, "normal"),
    ("q4hex_kappa_diff", 3, "QK", 4, 1, "IM_GAUSS_PARALLELEPIPED(3,9)", 2,
     "kappa*Grad_u.Grad_u", "kappa*Grad_u.Grad_u", {}, {"kappa": "P0"}, False, "normal"),
    ("q1hex_kappa_nodal_diff", 3, "QK", 1, 1, "IM_GAUSS_PARALLELEPIPED(3,3)", 3,
     "kappa*Grad_u.Grad_u", "kappa*Grad_u.Grad_u", {}, {"kappa": "S"}, True, "normal"),
    ("q2hex_nh_mu_diff", 3, "QK", 2, 3, "IM_GAUSS_PARALLELEPIPED(3,5)", 3,
     NH_EXPLICIT, NH_POT, {"D1": "C"}, {"mu": "P0"}, True, "modes"),
    ("p2tet_nh_mu_diff", 3, "PK", 2, 3, "IM_TETRAHEDRON(5)", 2,
     NH_EXPLICIT, NH_POT, {"D1": "C"}, {"mu": "P0"}, True, "modes"),
]


def sinusoid_modes(xyz: np.ndarray, qdim: int, rng) -> np.ndarray:
    """u_a(x) = sum of 8 modes 0.05 sin(k.x + phi), k ~ U[-pi,pi]^3."""
    u = np.zeros((xyz.shape[0], qdim))
    for a in range(qdim):
        for _ in range(8):
            k = rng.uniform(-np.pi, np.pi, xyz.shape[1])
            ph = rng.uniform(0, 2 * np.pi)
            u[:, a] += 0.05 * np.sin(xyz @ k + ph)
    return u.ravel()


def make_case(case, seed):
    name, dim, gt, deg, qdim, im, nx, expr, consts, jitter, ukind = case
    import getfem_gb300 as g
    rng = np.random.default_rng(seed)
    kind = "simplex" if gt == "PK" else "hex"
    h = 1.0 / nx
    jit = None
    if jitter:
        jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** dim, dim))
    mesh = g.Mesh.regular_unit(dim, nx, kind, jitter=jit)
    mf = g.MeshFem(mesh, qdim, degree=deg)
    ndof = mf.nb_dof()
    E = mesh.nb_convex()
    inputs = {}
    if ukind == "modes":
        inputs["u"] = sinusoid_modes(mf.basic_dof_nodes(), qdim, rng)
    elif ukind == "zero":
        inputs["u"] = np.zeros(ndof)
    else:
        inputs["u"] = rng.standard_normal(ndof) * 0.1
    for cname, ck in consts.items():
        if ck == "P0":
            sigma = 0.3 if cname == "mu" and ukind == "modes" else 0.2
            inputs[cname] = np.exp(rng.normal(0.0, sigma, E))
        elif ck == "V":
            inputs[cname] = rng.standard_normal(ndof) if qdim > 1 else rng.uniform(-1, 1, ndof)
        elif ck == "S":
            sigma = 0.3 if cname == "mu" and ukind == "modes" else 0.2
            inputs[cname] = np.exp(rng.normal(0.0, sigma, ndof // qdim))
        elif ck == "C":
            # Cani: a stiffness, stored in GetFEM's (Fortran) component order
            inputs[cname] = (stiffness_tensor(rng).ravel(order="F") if cname == "Cani"
                             else np.array([1.5]))
    with tempfile.TemporaryDirectory() as td:
        ind = os.path.join(td, "in")
        outd = os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        for k, v in inputs.items():
            np.asarray(v, dtype=np.float64).tofile(os.path.join(ind, k + ".bin"))
        if jit is not None:
            jit.astype(np.float64).tofile(os.path.join(ind, "jitter.bin"))
        cs = ",".join(f"{k}:{v}" for k, v in consts.items())
        cmd = [DRIVER, f"dim={dim}", f"nx={nx}", f"gt={gt}", f"fem={deg}", f"qdim={qdim}",
               f"im={im}", f"in={ind}", f"out={outd}", f"expr={expr}",
               f"orders={ORDERS.get(name, '2,1')}"] + EXTRA.get(name, []) + [
               f"jitter={1 if jit is not None else 0}", f"consts={cs}"]
        subprocess.run(cmd, check=True)
        info = json.load(open(os.path.join(outd, "info.json")))

        def rd(fn, dt=np.float64):
            return np.fromfile(os.path.join(outd, fn), dtype=dt)
        rec = dict(
            points=rd("points.bin").reshape(-1, dim),
            cvpts=rd("cvpts.bin", np.int64).reshape(E, -1),
            dofs=rd("dofs.bin", np.int64).reshape(E, -1),
            dofs0=rd("dofs0.bin", np.int64),
            im_points=rd("im_points.bin").reshape(-1, dim),
            im_weights=rd("im_weights.bin"),
            base_val=rd("base_val.bin"),
            base_grad=rd("base_grad.bin"),
            K_rowptr=rd("K_rowptr.bin", np.int64),
            K_colidx=rd("K_colidx.bin", np.int64).astype(np.int32),
            K_vals=rd("K_vals.bin"),
            R=rd("R.bin"),
        )
        if os.path.exists(os.path.join(outd, "E.bin")):
            rec["E"] = rd("E.bin")
        if os.path.exists(os.path.join(outd, "x.bin")):
            rec["x"] = rd("x.bin")
            rec["dirichlet"] = rd("dirichlet.bin", np.int64)
            rec["cg_iterations"] = np.array([info["cg_iterations"]])
    for k, v in inputs.items():
        rec["in_" + k] = np.asarray(v, dtype=np.float64)
    if jit is not None:
        rec["jitter"] = jit
    meta = dict(name=name, dim=dim, gt=gt, degree=deg, qdim=qdim, im=im, nx=nx, expr=expr,
                consts=consts, n_dof=info["n_dof"], nnz=info["nnz"], seed=seed)
    rec["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "ndof", info["n_dof"], "nnz", info["nnz"])


def make_diff_case(case, seed):
    """Energy and first derivatives (u and the coefficient declared as a
    variable) of a potential, from the reference's own symbolic derivative."""
    name, dim, gt, deg, qdim, im, nx, expr, gpu_expr, consts, varsd, jitter, ukind = case
    import getfem_gb300 as g
    rng = np.random.default_rng(seed)
    kind = "simplex" if gt == "PK" else "hex"
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** dim, dim)) if jitter else None
    mesh = g.Mesh.regular_unit(dim, nx, kind, jitter=jit)
    mf = g.MeshFem(mesh, qdim, degree=deg)
    ndof, E = mf.nb_dof(), mesh.nb_convex()
    inputs = {"u": (sinusoid_modes(mf.basic_dof_nodes(), qdim, rng) if ukind == "modes"
                    else rng.standard_normal(ndof) * 0.1)}
    for cname, ck in consts.items():
        inputs[cname] = np.array([1.5])
    for vname, vk in varsd.items():
        n = E if vk == "P0" else ndof // qdim
        sigma = 0.3 if vname == "mu" else 0.5
        inputs[vname] = np.exp(rng.normal(0.0, sigma, n))
    out = {}
    for tag, ex, vars_, orders in (("ref", expr, varsd, "0,1"), ("builtin", gpu_expr, {}, "0")):
        with tempfile.TemporaryDirectory() as td:
            ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
            os.makedirs(ind)
            os.makedirs(outd)
            for k, v in inputs.items():
                np.asarray(v, dtype=np.float64).tofile(os.path.join(ind, k + ".bin"))
            if jit is not None:
                jit.astype(np.float64).tofile(os.path.join(ind, "jitter.bin"))
            cs = dict(consts)
            if tag == "builtin":
                cs.update(varsd)  # the coefficient as a constant
            cmd = [DRIVER, f"dim={dim}", f"nx={nx}", f"gt={gt}", f"fem={deg}", f"qdim={qdim}",
                   f"im={im}", f"in={ind}", f"out={outd}", f"expr={ex}", f"orders={orders}",
                   f"jitter={1 if jit is not None else 0}",
                   "consts=" + ",".join(f"{k}:{v}" for k, v in cs.items()),
                   "vars=" + ",".join(f"{k}:{v}" for k, v in vars_.items())]
            subprocess.run(cmd, check=True)
            out[tag] = {fn[:-4]: np.fromfile(os.path.join(outd, fn))
                        for fn in ("E.bin", "R.bin") if os.path.exists(os.path.join(outd, fn))}
    E_ref, E_bi = float(out["ref"]["E"][0]), float(out["builtin"]["E"][0])
    assert abs(E_ref - E_bi) <= 1e-13 * abs(E_bi), (name, E_ref, E_bi)
    V = out["ref"]["R"]
    rec = {"E": np.array([E_ref]), "E_builtin": np.array([E_bi]), "dE_du": V[:ndof]}
    off = ndof
    for vname in varsd:
        n = inputs[vname].size
        rec["dE_d" + vname] = V[off:off + n]
        off += n
    assert off == V.size
    for k, v in inputs.items():
        rec["in_" + k] = np.asarray(v, dtype=np.float64)
    if jit is not None:
        rec["jitter"] = jit
    meta = dict(name=name, dim=dim, gt=gt, degree=deg, qdim=qdim, im=im, nx=nx, expr=expr,
                gpu_expr=gpu_expr, consts=consts, vars=varsd, n_dof=ndof, seed=seed)
    rec["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "E", E_ref, "vars", list(varsd))


def make_condensed_case(case, seed):
    """The reference's assembly(1, true) and assembly(2, true) over a model
    holding u and the internal variable p (ref_driver internal=p)."""
    name, dim, gt, deg, qdim, im, nx, expr_a, expr_b, consts, jitter = case
    import getfem_gb300 as g
    rng = np.random.default_rng(seed)
    kind = "simplex" if gt == "PK" else "hex"
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** dim, dim)) if jitter else None
    mesh = g.Mesh.regular_unit(dim, nx, kind, jitter=jit)
    mf = g.MeshFem(mesh, qdim, degree=deg)
    ndof, E = mf.nb_dof(), mesh.nb_convex()
    nq = g.MeshIm(mesh, im).nq
    inputs = {"u": rng.standard_normal(ndof) * 0.05, "p": rng.standard_normal(E * nq) * 0.05}
    for cname, ck in consts.items():
        inputs[cname] = np.exp(rng.normal(0.0, 0.2, E)) if ck == "P0" else np.array([1.5])
    with tempfile.TemporaryDirectory() as td:
        ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        for k, v in inputs.items():
            np.asarray(v, dtype=np.float64).tofile(os.path.join(ind, k + ".bin"))
        if jit is not None:
            jit.astype(np.float64).tofile(os.path.join(ind, "jitter.bin"))
        cs = ",".join(f"{k}:{v}" for k, v in consts.items())
        cmd = [DRIVER, f"dim={dim}", f"nx={nx}", f"gt={gt}", f"fem={deg}", f"qdim={qdim}",
               f"im={im}", f"in={ind}", f"out={outd}", f"expr={expr_a}", f"expr2={expr_b}",
               "internal=p", f"jitter={1 if jit is not None else 0}", f"consts={cs}"]
        subprocess.run(cmd, check=True)
        info = json.load(open(os.path.join(outd, "info.json")))

        def rd(fn, dt=np.float64):
            return np.fromfile(os.path.join(outd, fn), dtype=dt)
        rec = dict(
            points=rd("points.bin").reshape(-1, dim),
            cvpts=rd("cvpts.bin", np.int64).reshape(E, -1),
            dofs=rd("dofs.bin", np.int64).reshape(E, -1),
            R_full=rd("R_full.bin"),
            K_rowptr=rd("K_rowptr.bin", np.int64),
            K_colidx=rd("K_colidx.bin", np.int64).astype(np.int32),
            K_vals=rd("K_vals.bin"),
            Rc=rd("Rc.bin"),
            C_rowptr=rd("C_rowptr.bin", np.int64),
            C_colidx=rd("C_colidx.bin", np.int64).astype(np.int32),
            C_vals=rd("C_vals.bin"),
        )
    for k, v in inputs.items():
        rec["in_" + k] = np.asarray(v, dtype=np.float64)
    if jit is not None:
        rec["jitter"] = jit
    meta = dict(name=name, dim=dim, gt=gt, degree=deg, qdim=qdim, im=im, nx=nx, expr=expr_a,
                expr2=expr_b, consts=consts, n_dof=info["n_dof"], nnz=info["nnz"],
                n_internal=info["n_internal"], seed=seed)
    assert info["n_internal"] == E * nq
    rec["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "ndof", info["n_dof"], "nnz", info["nnz"], "internal", info["n_internal"])


def main():
    if not os.path.exists(DRIVER):
        sys.exit(f"{DRIVER} missing: build it with make -C oracle/refbuild")
    only = set(sys.argv[1:])  # optional: names of the fixtures to (re)make
    for i, case in enumerate(CASES):
        if not only or case[0] in only:
            make_case(case, 1000 + i)
    for i, case in enumerate(CONDENSE_CASES):
        if not only or case[0] in only:
            make_condensed_case(case, 2000 + i)
    for i, case in enumerate(DIFF_CASES):
        if not only or case[0] in only:
            make_diff_case(case, 4000 + i)


if __name__ == "__main__":
    main()
