"""The GetFEM-side drop-in (getfem_gb300/getfem_shim): the C++ lowering that
walks the reference's analysed GWFL trees, and getfem::ga_workspace::assembly
on the GPU linked ahead of the reference's own definition.

CPU: for every expression of the reference fixtures the C++ lowering (run on
the trees the reference's add_expression built) and the Python front end
(getfem_gb300.gwfl) give the same descriptor terms for orders 0, 1 and 2, and
both reject the same unsupported expressions.

GPU: the reference's own fixture driver (oracle/refbuild/ref_driver.cc),
linked with the drop-in, assembles the fixtures through unchanged
ga_workspace::assembly calls and through model::assembly with several
OpenMP threads (each thread's workspace holds its partition of the mesh),
and gets the reference's K and R (pattern bit-exact, values within 1e-12);
an unsupported expression fails with the drop-in's error."""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L

from common import (GOLDEN, RTOL, assert_same_pattern, build_case, golden_csr, golden_names,
                    load, value_errors, vec_errors)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM_TESTS = os.path.join(ROOT, "tests", "shim")
ARCH = os.uname().machine
OUT = os.path.join(ROOT, "oracle", "_ref", "shim-" + ARCH)


def _reference_available():
    return os.path.exists(os.path.join(ROOT, "oracle", "_ref", f"libgetfem_ref-{ARCH}.a"))


def _build(target):
    if not _reference_available():
        pytest.skip("the reference GetFEM build (oracle/_ref) is absent")
    r = subprocess.run(["make", "-C", SHIM_TESTS, target], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]


# ----------------------------------------------------------- lowering (CPU)

def _data_spec(rec):
    m = rec["meta"]
    out = []
    for name, kind in m["consts"].items():
        if kind == "C":
            vals = ";".join(repr(float(x)) for x in np.atleast_1d(rec["in_" + name]))
            out.append(f"{name}:C={vals}")
        else:
            out.append(f"{name}:{kind}")
    return ",".join(out)


def _cpp_lower(cases):
    """cases: list of (name, dim, nx, gt, degree, qdim, im, expr, data spec)."""
    _build("all")
    lines = "\n".join("|".join(str(x) for x in c) for c in cases) + "\n"
    r = subprocess.run([os.path.join(OUT, "lower_check")], input=lines, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = {}
    for ln in r.stdout.splitlines():
        d = json.loads(ln)
        out[(d["name"], d["order"])] = d
    return out


def _canon(kind, scale, field, coefs, tensor=None):
    """A term with the overall scale folded into the coefficients of the
    GRADGRAD and MASS terms (scale 2, value 1 is the same term as scale 1,
    value 2); a GRADGRAD_TENSOR term carries its tensor (padded to
    GFGPU_MAX_TENSOR entries)."""
    if kind in (L.TERM_GRADGRAD, L.TERM_MASS):
        coefs = [(k, v * scale if k else 0.0, d) for k, v, d in coefs]
        scale = 1.0
    ten = ()
    if kind == L.TERM_GRADGRAD_TENSOR:
        t = list(tensor) + [0.0] * (L.MAX_TENSOR - len(tensor))
        ten = tuple(round(float(x), 12) for x in t)
    return (kind, round(scale, 12), field,
            tuple((k, round(v, 12), d) for k, v, d in coefs), ten)


def _canon_cpp(forms):
    terms = []
    for f in forms:
        for t in f["terms"]:
            terms.append(_canon(t["kind"], t["scale"], t["field"],
                                [(c["kind"], c["value"], c["data"]) for c in t["c"]],
                                t.get("tensor")))
    return sorted(terms)


def _canon_py(ws, terms):
    by_slot = {d.slot: name for name, d in ws.data.items() if d.slot >= 0}
    out = []
    for t in terms:
        cs = []
        for c in t["c"]:
            if c is None or c["kind"] == L.COEF_NONE:
                cs.append((0, 0.0, ""))
            else:
                data = by_slot[c["slot"]] if c["kind"] in (L.COEF_ELEMENT, L.COEF_NODAL) else ""
                cs.append((c["kind"], c["value"], data))
        field = by_slot[t["field_slot"]] if t["kind"] == L.TERM_SOURCE else ""
        out.append(_canon(t["kind"], t["scale"], field, cs, t.get("tensor")))
    return sorted(out)


def _fixture_cases():
    cases = []
    for name in golden_names():
        rec = load(name)
        m = rec["meta"]
        cases.append((name, m["dim"], 2, m["gt"], m["degree"], m["qdim"], m["im"], m["expr"],
                      _data_spec(rec)))
    return cases


def test_cpp_lowering_equals_python_lowering_on_every_fixture():
    cases = _fixture_cases()
    cpp = _cpp_lower(cases)
    for c in cases:
        name = c[0]
        rec = load(name)
        mesh, mf, mim, ws = build_case(rec)
        grp = ws.groups[0]
        for order, terms in ((0, grp.order0), (1, grp.order1), (2, grp.order2)):
            d = cpp[(name, order)]
            assert "error" not in d, (name, order, d["error"])
            assert _canon_cpp(d["forms"]) == _canon_py(ws, terms), (name, order)


UNSUPPORTED = [
    # (name, dim, gt, degree, qdim, im, expr, data)
    ("norm", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "Norm(Grad_u)*Test_u", ""),
    ("u_squared", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "u*u*Test_u", ""),
    ("u_grad", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "u*Grad_u.Grad_Test_u", ""),
    ("position", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "X(1)*Grad_u.Grad_Test_u", ""),
    ("sin_of_data", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "sin(kappa)*Grad_u.Grad_Test_u", "kappa:P0"),
    ("data_squared", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "kappa*kappa*Grad_u.Grad_Test_u", "kappa:P0"),
    ("value_gradient", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "Grad_u(1)*Test_u", ""),
    ("anisotropic_unsymmetric", 3, "PK", 1, 3, "IM_TETRAHEDRON(2)",
     "Grad_u(1,2)*Grad_Test_u(1,1)", ""),
    ("anisotropic_potential", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "([2,0.5;0.5,1]*Grad_u).Grad_u", ""),
    ("two_anisotropic_sources", 2, "PK", 1, 1, "IM_TRIANGLE(2)",
     "kappa*([2,0;0,1]*Grad_u).Grad_Test_u + ([1,0.5;0.5,1]*Grad_u).Grad_Test_u", "kappa:P0"),
    ("constant_source", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "Grad_u.Grad_Test_u - 3*Test_u", ""),
    ("gradient_source", 2, "PK", 1, 1, "IM_TRIANGLE(2)", "Grad_u.Grad_Test_u - Grad_f.Grad_Test_u",
     "f:V"),
    ("det", 3, "PK", 1, 3, "IM_TETRAHEDRON(2)", "Det(Id(3)+Grad_u)*Div_Test_u", ""),
]


def _py_rejects(case):
    name, dim, gt, deg, qdim, im, expr, data = case
    mesh = g.Mesh.regular_unit(dim, 2, "simplex" if gt == "PK" else "hex")
    mf = g.MeshFem(mesh, qdim, degree=deg)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    for spec in filter(None, data.split(",")):
        nm, k = spec.split(":")
        if k == "P0":
            ws.add_fem_constant(nm, g.MeshFem(mesh, 1, degree=0), np.ones(mesh.nb_convex()))
        elif k == "V":
            ws.add_fem_constant(nm, mf, np.ones(mf.nb_dof()))
    try:
        ws.add_expression(expr, g.MeshIm(mesh, im))
    except L.UnsupportedExpression:
        return True
    return False


def test_cpp_and_python_reject_the_same_expressions():
    cases = [(c[0], c[1], 2, c[2], c[3], c[4], c[5], c[6], c[7]) for c in UNSUPPORTED]
    cpp = _cpp_lower(cases)
    for c in UNSUPPORTED:
        rejected_cpp = any("error" in cpp[(c[0], o)] for o in (0, 1, 2))
        assert rejected_cpp, (c[0], [cpp[(c[0], o)] for o in (0, 1, 2)])
        assert _py_rejects(c), c[0]


def _stiffness81():
    """A 3-D stiffness with major and minor symmetry, Fortran order."""
    rng = np.random.default_rng(8)
    M = rng.uniform(-0.3, 0.3, (6, 6))
    S = (M + M.T) / 2 + np.diag(rng.uniform(1.0, 3.0, 6))
    V = [[0, 5, 4], [5, 1, 3], [4, 3, 2]]
    C = np.zeros((3, 3, 3, 3))
    for a in range(3):
        for k in range(3):
            for b in range(3):
                for l in range(3):
                    C[a, k, b, l] = S[V[a][k], V[b][l]]
    return C.ravel(order="F")


def _cspec(name, vals):
    return f"{name}:C=" + ";".join(repr(float(x)) for x in vals)


TRI = (2, "PK", 1, 1, "IM_TRIANGLE(2)")
TET3 = (3, "PK", 1, 3, "IM_TETRAHEDRON(2)")
# spellings beyond the fixtures: (name, space, expr, data)
SPELLINGS = [
    ("lap_swapped", TRI, "Grad_Test_u.Grad_u", ""),
    ("lap_scaled", TRI, "2*Grad_u.Grad_Test_u - 0.5*Grad_Test_u.Grad_u", ""),
    ("kappa_inside", TRI, "(kappa*Grad_u).Grad_Test_u", "kappa:P0"),
    ("kappa_right", TRI, "Grad_u.Grad_Test_u*kappa", "kappa:P0"),
    ("mass_lap", TRI, "u*Test_u*3 + Grad_u.Grad_Test_u", ""),
    ("aniso_literal", TRI, "([2,0.5;0.5,1]*Grad_u).Grad_Test_u", ""),
    ("aniso_swapped", TRI, "Grad_Test_u.([2,0.5;0.5,1]*Grad_u)", ""),
    ("aniso_tensor_product", TRI, "[2,0.5;0.5,1]:(Grad_u@Grad_Test_u)", ""),
    ("aniso_reshaped_data", TRI, "(Reshape(A,2,2)*Grad_u).Grad_Test_u",
     _cspec("A", [2.0, 0.5, 0.5, 1.0])),
    ("aniso_kappa_plus_iso", TRI,
     "kappa*([3,1;1,2]*Grad_u).Grad_Test_u + Grad_u.Grad_Test_u - f*Test_u", "kappa:P0,f:V"),
    ("potential_mass_lap", TRI, "kappa*Grad_u.Grad_u + u*u", "kappa:P0"),
    ("elastic_div", TET3, "lambda*Div_u*Div_Test_u + 2*mu*Sym(Grad_u):Grad_Test_u",
     "lambda:P0,mu:P0"),
    ("elastic_trace", TET3, "(lambda*Trace(Grad_u)*Id(3) + mu*(Grad_u+Grad_u')):Grad_Test_u",
     "lambda:P0,mu:P0"),
    ("elastic_sym_test", TET3, "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Sym(Grad_Test_u)",
     "lambda:P0,mu:P0"),
    ("deviator", TET3, "Deviator(Sym(Grad_u)):Grad_Test_u", ""),
    ("aniso_stiffness", TET3, "(Reshape(Cani,3,3,3,3):Grad_u):Grad_Test_u - f.Test_u",
     _cspec("Cani", _stiffness81()) + ",f:V"),
    ("aniso_separable", TET3,
     "([2,0,0;0,1,0;0,0,1]*Grad_u*[1,0.5,0;0.5,1,0;0,0,1]):Grad_Test_u", ""),
]


def _py_ws(space, expr, data):
    dim, gt, deg, qdim, im = space
    mesh = g.Mesh.regular_unit(dim, 2, "simplex" if gt == "PK" else "hex")
    mf = g.MeshFem(mesh, qdim, degree=deg)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    for spec in filter(None, data.split(",")):
        nm, k = spec.split(":", 1)
        if k == "P0":
            ws.add_fem_constant(nm, g.MeshFem(mesh, 1, degree=0), np.ones(mesh.nb_convex()))
        elif k == "V":
            ws.add_fem_constant(nm, mf, np.ones(mf.nb_dof()))
        elif k.startswith("C="):
            ws.add_fixed_size_constant(nm, np.array([float(x) for x in k[2:].split(";")]))
    ws.add_expression(expr, g.MeshIm(mesh, im))
    return ws


def test_cpp_and_python_lowerings_agree_on_more_spellings():
    cases = [(nm, sp[0], 2, sp[1], sp[2], sp[3], sp[4], expr, data)
             for nm, sp, expr, data in SPELLINGS]
    cpp = _cpp_lower(cases)
    for nm, sp, expr, data in SPELLINGS:
        ws = _py_ws(sp, expr, data)
        grp = ws.groups[0]
        for order, terms in ((0, grp.order0), (1, grp.order1), (2, grp.order2)):
            d = cpp[(nm, order)]
            assert "error" not in d, (nm, order, d["error"])
            assert _canon_cpp(d["forms"]) == _canon_py(ws, terms), (nm, order)


def _random_forms(n, seed=31):
    """Seeded random weak forms built from the lowered families, with dyadic
    coefficients (exact in both lowerings): (name, space, expr, data)."""
    rng = np.random.default_rng(seed)

    def c():
        return f"{int(rng.integers(1, 16)) / 8:g}"
    out = []
    for i in range(n):
        if i % 2 == 0:
            dim = int(rng.choice([2, 3]))
            space = TRI if dim == 2 else (3, "PK", 1, 1, "IM_TETRAHEDRON(2)")
            parts = [f"{c()}*Grad_u.Grad_Test_u"]
            if rng.random() < 0.5:
                parts.append(f"kappa*Grad_u.Grad_Test_u*{c()}")
            if rng.random() < 0.5:
                parts.append(f"{c()}*u*Test_u")
            if rng.random() < 0.6:
                M = rng.integers(-4, 5, (dim, dim)) / 4
                A = M + M.T + np.eye(dim) * 3
                lit = ";".join(",".join(f"{x:g}" for x in row) for row in A)
                scale = "kappa*" if rng.random() < 0.5 and "kappa" not in " ".join(parts) else ""
                parts.append(f"{scale}([{lit}]*Grad_u).Grad_Test_u")
            if rng.random() < 0.5:
                parts.append("- f*Test_u")
        else:
            space = TET3
            parts = [f"{c()}*Div_u*Div_Test_u"]
            for t in ("Sym(Grad_u):Grad_Test_u", "Grad_u:Grad_Test_u", "Grad_u':Grad_Test_u",
                      "lambda*Div_u*Div_Test_u", "mu*(Grad_u+Grad_u'):Grad_Test_u", "u.Test_u"):
                if rng.random() < 0.4:
                    parts.append(f"{c()}*{t}")
            if rng.random() < 0.3:
                parts.append("([2,0,0;0,1,0;0,0,1]*Grad_u*[1,0.5,0;0.5,1,0;0,0,1]):Grad_Test_u")
            if rng.random() < 0.5:
                parts.append("- f.Test_u")
        expr = " + ".join(parts).replace("+ -", "-")
        used = [d for d in ("kappa", "lambda", "mu") if d in expr]
        has_f = "f*Test_u" in expr or "f.Test_u" in expr
        data = ",".join([f"{d}:P0" for d in used] + (["f:V"] if has_f else []))
        out.append((f"random_{i}", space, expr, data))
    return out


def test_cpp_and_python_lowerings_agree_on_random_forms():
    forms = _random_forms(24)
    cases = [(nm, sp[0], 2, sp[1], sp[2], sp[3], sp[4], expr, data)
             for nm, sp, expr, data in forms]
    cpp = _cpp_lower(cases)
    for nm, sp, expr, data in forms:
        ws = _py_ws(sp, expr, data)
        grp = ws.groups[0]
        for order, terms in ((1, grp.order1), (2, grp.order2)):
            d = cpp[(nm, order)]
            assert "error" not in d, (nm, expr, order, d["error"])
            assert _canon_cpp(d["forms"]) == _canon_py(ws, terms), (nm, expr, order)


# ------------------------------------------------------- drop-in (GPU)

def _run_shim(rec, orders="2,1", extra=()):
    m = rec["meta"]
    _build("gpu")
    with tempfile.TemporaryDirectory() as td:
        ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        for k in rec:
            if k.startswith("in_"):
                np.asarray(rec[k], dtype=np.float64).tofile(os.path.join(ind, k[3:] + ".bin"))
        if "jitter" in rec:
            np.asarray(rec["jitter"], dtype=np.float64).tofile(os.path.join(ind, "jitter.bin"))
        cmd = [os.path.join(OUT, "shim_driver"), f"dim={m['dim']}", f"nx={m['nx']}",
               f"gt={m['gt']}", f"fem={m['degree']}", f"qdim={m['qdim']}", f"im={m['im']}",
               f"in={ind}", f"out={outd}", f"expr={m['expr']}", f"orders={orders}",
               f"jitter={1 if 'jitter' in rec else 0}", "dump=0",
               "consts=" + ",".join(f"{k}:{v}" for k, v in m["consts"].items())] + list(extra)
        r = subprocess.run(cmd, capture_output=True, text=True)
        res = {"rc": r.returncode, "err": r.stderr + r.stdout}
        for fn in ("K_rowptr", "K_colidx", "K_vals", "R", "rhs", "E"):
            p = os.path.join(outd, fn + ".bin")
            if os.path.exists(p):
                res[fn] = np.fromfile(p, dtype=np.int64 if fn in ("K_rowptr", "K_colidx")
                                      else np.float64)
    return res


def _csr(res, n):
    import scipy.sparse as sp
    return sp.csr_matrix((res["K_vals"], res["K_colidx"].astype(np.int32), res["K_rowptr"]),
                         shape=(n, n))


SHIM_CASES = ["p1tri_poisson", "p2tri_elastic", "p2tet_elastic", "q2hex_elastic_nodal",
              "q2hex_neohookean", "q4hex_laplace", "q1hex_nodal_kappa", "p2tet_aniso_elastic"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", SHIM_CASES)
def test_dropin_workspace_assembly_matches_reference(name):
    rec = load(name)
    res = _run_shim(rec)
    assert res["rc"] == 0, res["err"][-2000:]
    K = _csr(res, rec["meta"]["n_dof"])
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    assert vec_errors(res["R"], rec["R"]).max() <= RTOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["p2tet_elastic", "q2hex_neohookean", "q4hex_laplace",
                                  "q1hex_nodal_kappa"])
def test_dropin_model_assembly_with_threads_matches_reference(name):
    """model::assembly(BUILD_ALL) with 4 OpenMP threads: each thread's
    workspace assembles its partition of the mesh on the GPU; the model sums
    the partitions (accumulated_distro)."""
    rec = load(name)
    res = _run_shim(rec, extra=["time=model", "threads=4", "warmup=0", "steps=1",
                                "model_out=1"])
    assert res["rc"] == 0, res["err"][-2000:]
    K = _csr(res, rec["meta"]["n_dof"])
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    assert vec_errors(-res["rhs"], rec["R"]).max() <= RTOL


@pytest.mark.gpu
def test_dropin_rejects_an_unsupported_expression():
    rec = dict(load("p1tri_poisson"))
    meta = dict(rec["meta"])
    meta["expr"] = "Norm(Grad_u)*Test_u"
    meta["consts"] = {}
    rec["meta"] = meta
    res = _run_shim(rec, orders="1")
    assert res["rc"] != 0
    assert "not lowered for the GPU" in res["err"]
