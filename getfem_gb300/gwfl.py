"""GWFL front end for the GPU backend: parser, numeric evaluator, lowering.

GetFEM compiles a GWFL string in three steps: ga_read_string builds a tree
(src/getfem_generic_assembly_tree.cc), ga_semantic_analysis types it
(src/getfem_generic_assembly_semantic.cc:2708) and ga_workspace::add_tree
derives it symbolically up to order 2 (src/getfem_generic_assembly_workspace.cc:439-543).
This module covers the part of that language the GPU kernels execute and
lowers an expression to the descriptor of include/gfgpu.h:

  * the tokenizer/parser follows GWFL's operator priorities
    (getfem_generic_assembly_tree.cc:50-66): '+' '-' < '*' '/' ':' '.' '.*'
    './' '@' < unary '-' and transpose "'" < Sym/Skew/Trace/Deviator;
  * the evaluator implements the tensor semantics of those operators with
    numpy on one integration point;
  * lowering probes the integrand numerically.  An order-1 weak form that is
    affine in the variable, R(u; v) = a(u, v) - l(v), is identified by
    evaluating it on unit test/trial tensors; a(u, v) must be an isotropic
    gradient coupling D = c0 d_ak d_bl + c1 d_ab d_kl + c2 d_al d_kb plus a
    mass term, each coefficient linear in the data fields, to which one
    constant symmetric anisotropic coupling D[(a,k),(b,l)] may be added
    (times a constant or one per-element field: (A*Grad_u).Grad_Test_u,
    (Reshape(C,3,3,3,3):Grad_u):Grad_Test_u); l must be a
    field on the variable's mesh_fem times a constant.  Alternative
    spellings of the same weak form therefore lower identically, as the
    reference's own tests require of the CPU compiler
    (tests/test_assembly.cc:773-882).
  * the finite-strain hyperelasticity brick form
    ((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[C1;D1]))):Grad_Test_u
    (src/getfem_nonlinear_elasticity.cc:2319-2320) is matched by structure.

Anything else raises UnsupportedExpression when the expression is added:
there is no CPU fallback.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

# ------------------------------------------------------------------ parser

_TOKEN = re.compile(r"""
    (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?)
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>\.\*|\./|:=|[-+*/:.@'(),;\[\]])
  | (?P<ws>\s+)
""", re.VERBOSE)


@dataclass
class Node:
    kind: str                 # num, name, call, bin, neg, quote, matrix
    value: object = None      # number, name, operator
    args: list = field(default_factory=list)

    def __repr__(self):
        if self.kind == "num":
            return repr(self.value)
        if self.kind == "name":
            return str(self.value)
        if self.kind == "call":
            return f"{self.value}({', '.join(map(repr, self.args))})"
        if self.kind == "bin":
            return f"({self.args[0]!r} {self.value} {self.args[1]!r})"
        if self.kind == "neg":
            return f"(-{self.args[0]!r})"
        if self.kind == "quote":
            return f"{self.args[0]!r}'"
        return "[" + "; ".join(", ".join(map(repr, r)) for r in self.args) + "]"


class ParseError(L.UnsupportedExpression):
    def __init__(self, msg):
        super().__init__(L.E_UNSUPPORTED, msg)


def tokenize(s: str):
    toks = []
    pos = 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise ParseError(f"GWFL: unexpected character {s[pos]!r} at {pos} in {s!r}")
        pos = m.end()
        if m.lastgroup == "ws":
            continue
        toks.append((m.lastgroup, m.group(m.lastgroup)))
    toks.append(("end", None))
    return toks


_BINARY = {"+": 1, "-": 1, "*": 2, "/": 2, ":": 2, ".": 2, ".*": 2, "./": 2, "@": 2}


class _Parser:
    def __init__(self, s):
        self.t = tokenize(s)
        self.i = 0
        self.s = s

    def peek(self):
        return self.t[self.i]

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise ParseError(f"GWFL: expected {val!r}, got {tok[1]!r} in {self.s!r}")
        self.i += 1
        return tok

    def parse(self):
        n = self.expr(1)
        if self.peek()[0] != "end":
            raise ParseError(f"GWFL: trailing input {self.peek()[1]!r} in {self.s!r}")
        return n

    def expr(self, minprio):
        lhs = self.unary()
        while True:
            kind, val = self.peek()
            if kind != "op" or val not in _BINARY or _BINARY[val] < minprio:
                return lhs
            self.take()
            rhs = self.expr(_BINARY[val] + 1)
            lhs = Node("bin", val, [lhs, rhs])

    def unary(self):
        kind, val = self.peek()
        if kind == "op" and val == "-":
            self.take()
            return Node("neg", None, [self.unary()])
        if kind == "op" and val == "+":
            self.take()
            return self.unary()
        return self.postfix()

    def postfix(self):
        n = self.primary()
        while self.peek() == ("op", "'"):
            self.take()
            n = Node("quote", None, [n])
        return n

    def primary(self):
        kind, val = self.take()
        if kind == "num":
            return Node("num", float(val))
        if kind == "name":
            if self.peek() == ("op", "("):
                self.take()
                args = []
                if self.peek() != ("op", ")"):
                    args.append(self.expr(1))
                    while self.peek() == ("op", ","):
                        self.take()
                        args.append(self.expr(1))
                self.take(")")
                return Node("call", val, args)
            return Node("name", val)
        if (kind, val) == ("op", "("):
            n = self.expr(1)
            self.take(")")
            return n
        if (kind, val) == ("op", "["):
            rows = [[self.expr(1)]]
            while self.peek()[1] in (",", ";"):
                sep = self.take()[1]
                if sep == ",":
                    rows[-1].append(self.expr(1))
                else:
                    rows.append([self.expr(1)])
            self.take("]")
            return Node("matrix", None, rows)
        raise ParseError(f"GWFL: unexpected token {val!r} in {self.s!r}")


def parse(s: str) -> Node:
    return _Parser(s).parse()


# ---------------------------------------------------------------- evaluator

def _contract(A, B, n):
    A = np.asarray(A)
    B = np.asarray(B)
    if A.ndim < n or B.ndim < n:
        raise ParseError("GWFL: contraction of tensors of too low order")
    return np.tensordot(A, B, axes=(list(range(A.ndim - n, A.ndim)), list(range(n))))


def _binop(op, a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    if op in "+-":
        if a.shape != b.shape:
            raise ParseError(f"GWFL: '{op}' of tensors of shapes {a.shape} and {b.shape}")
        return a + b if op == "+" else a - b
    if op == "*":
        if a.ndim == 0 or b.ndim == 0:
            return a * b
        if a.ndim == 2:
            return _contract(a, b, 1)
        raise ParseError(f"GWFL: '*' of shapes {a.shape} and {b.shape}")
    if op == "/":
        if b.ndim != 0:
            raise ParseError("GWFL: division by a non-scalar")
        return a / b
    if op == ".":
        return _contract(a, b, 1)
    if op == ":":
        if a.ndim < 2 or b.ndim < 2:
            raise ParseError("GWFL: ':' needs order >= 2 tensors")
        return _contract(a, b, 2)
    if op == ".*":
        return a * b
    if op == "./":
        return a / b
    if op == "@":
        return np.multiply.outer(a, b)
    raise ParseError(f"GWFL: operator {op}")


def _fun(name, args):
    a = [np.asarray(x, dtype=float) for x in args]
    if name == "Id":
        return np.eye(int(round(float(a[0]))))
    if name == "Trace":
        return np.trace(a[0])
    if name == "Sym":
        return 0.5 * (a[0] + a[0].T)
    if name == "Skew":
        return 0.5 * (a[0] - a[0].T)
    if name == "Deviator":
        n = a[0].shape[0]
        return a[0] - np.trace(a[0]) / n * np.eye(n)
    if name == "Det":
        return np.linalg.det(a[0])
    if name == "Inv":
        return np.linalg.inv(a[0])
    if name == "Norm":
        return np.sqrt(np.sum(a[0] * a[0]))
    if name == "Norm_sqr":
        return np.sum(a[0] * a[0])
    if name == "Transpose":
        return a[0].T
    if name == "Reshape":
        # components in Fortran order (first index fastest), as GetFEM
        # stores every tensor
        dims = [int(round(float(x))) for x in a[1:]]
        if not dims or int(np.prod(dims)) != a[0].size:
            raise ParseError("GWFL: Reshape to incompatible sizes")
        return np.reshape(a[0].ravel(order="F"), dims, order="F")
    if name == "sqr":
        return a[0] * a[0]
    if name == "pow":
        return a[0] ** a[1]
    fn = {"sqrt": np.sqrt, "exp": np.exp, "log": np.log, "sin": np.sin, "cos": np.cos,
          "tan": np.tan, "abs": np.abs}.get(name)
    if fn is not None:
        return fn(a[0])
    raise ParseError(f"GWFL: function or operator {name!r} is not lowered to the GPU")


_OPERATORS = {"Compressible_Neo_Hookean_PK2"}


def evaluate(n: Node, env: dict):
    k = n.kind
    if k == "num":
        return np.asarray(n.value)
    if k == "name":
        if n.value not in env:
            raise ParseError(f"GWFL: unknown name {n.value!r}")
        return np.asarray(env[n.value], dtype=float)
    if k == "neg":
        return -evaluate(n.args[0], env)
    if k == "quote":
        v = evaluate(n.args[0], env)
        return v.T if v.ndim == 2 else v
    if k == "bin":
        return _binop(n.value, evaluate(n.args[0], env), evaluate(n.args[1], env))
    if k == "call":
        if n.value in _OPERATORS:
            raise ParseError(f"GWFL: {n.value} only inside the hyperelasticity brick form")
        return _fun(n.value, [evaluate(a, env) for a in n.args])
    rows = [[evaluate(x, env) for x in r] for r in n.args]
    if all(len(r) == 1 for r in rows):
        return np.array([float(r[0]) for r in rows])
    return np.array([[float(x) for x in r] for r in rows])


def names_in(n: Node) -> set:
    out = set()
    if n.kind == "name":
        out.add(n.value)
    if n.kind == "call":
        out.add(n.value + "()")
    for a in n.args:
        if isinstance(a, list):
            for x in a:
                out |= names_in(x)
        else:
            out |= names_in(a)
    return out


# ----------------------------------------------------------------- lowering

@dataclass
class FieldInfo:
    """A named datum of the workspace as the lowering sees it."""
    name: str
    kind: str            # 'variable', 'element' (P0), 'nodal' (scalar field on
                         # the variable's scalar mesh_fem), 'vfield' (field on
                         # the variable's mesh_fem), 'const', 'internal' (an
                         # internal im_data variable, scalar per Gauss point)
    qdim: int = 1
    value: object = None  # for 'const': the numpy value
    slot: int = -1


@dataclass
class Lowered:
    """Descriptor terms of one expression, per assembly order."""
    order2: list          # list of term dicts (bilinear part)
    order1: list          # terms whose order-1 assembly gives the residual
    order0: list          # potential terms
    max_order: int
    # an internal variable's part of a displacement / pressure pair
    # (merged into one TERM_INTERNAL_P by the workspace): {'name', 'sp'} for
    # the u equation, {'name', 'scale', 'c3', 'kb'} for the p equation
    internal: dict = None


def _term(kind, scale=1.0, c=(None, None, None), field_slot=0):
    return {"kind": kind, "scale": scale, "field_slot": field_slot, "c": list(c)}


def _coef(kind, slot=0, value=1.0):
    return {"kind": kind, "slot": slot, "value": value}


class _Probe:
    """Numeric probing of a weak form on one integration point."""

    def __init__(self, tree, var, dim, fields):
        self.tree = tree
        self.var = var
        self.dim = dim
        self.Q = var.qdim
        self.fields = fields

    def env(self, U, GU, V, GV, V2=None, GV2=None, theta=None):
        Q, N = self.Q, self.dim
        name = self.var.name
        e = {"meshdim": float(N), "pi": math.pi, "qdim": float(Q)}

        def shaped(vec, grad):
            if Q == 1:
                return float(vec[0]), np.array(grad[0])
            return np.array(vec), np.array(grad)
        u, gu = shaped(U, GU)
        e[name] = u
        e["Grad_" + name] = gu
        if Q == N:
            e["Div_" + name] = float(np.trace(GU)) if Q > 1 else float(GU[0][0])
        if V is not None:
            v, gv = shaped(V, GV)
            e["Test_" + name] = v
            e["Grad_Test_" + name] = gv
            if Q == N:
                e["Div_Test_" + name] = float(np.trace(GV)) if Q > 1 else float(GV[0][0])
        if V2 is not None:
            v2, gv2 = shaped(V2, GV2)
            e["Test2_" + name] = v2
            e["Grad_Test2_" + name] = gv2
            if Q == N:
                e["Div_Test2_" + name] = float(np.trace(GV2)) if Q > 1 else float(GV2[0][0])
        for f in self.fields.values():
            if f.kind == "const":
                e[f.name] = f.value
            elif f.kind in ("element", "nodal", "internal"):
                e[f.name] = theta.get(f.name, 0.0)
            elif f.kind == "vfield":
                val = theta.get(f.name, np.zeros(f.qdim))
                e[f.name] = float(val[0]) if f.qdim == 1 else np.array(val)
        return e

    def eval(self, **kw):
        return float(evaluate(self.tree, self.env(**kw)))


def _basis(Q, N):
    """Unit value tensors (Q) and unit gradient tensors (Q x N)."""
    vals = []
    for a in range(Q):
        v = np.zeros(Q)
        v[a] = 1
        vals.append(v)
    grads = []
    for a in range(Q):
        for k in range(N):
            g = np.zeros((Q, N))
            g[a, k] = 1
            grads.append(g)
    return vals, grads


def _iso_fit(D, Q, N):
    """Read D[(a,k),(b,l)] = c0 d_ak d_bl + c1 d_ab d_kl + c2 d_al d_kb off
    the entries where a single coefficient appears, then check every entry."""
    if Q == 1:
        c = np.array([0.0, D[0, 0], 0.0])
    else:
        c = np.array([D[0 * N + 0, 1 * N + 1],   # a=k=0, b=l=1: c0 only
                      D[0 * N + 1, 0 * N + 1],   # a=b=0, k=l=1: c1 only
                      D[0 * N + 1, 1 * N + 0]])  # a=0,k=1,b=1,l=0: c2 only
    err = 0.0
    for a in range(Q):
        for k in range(N):
            for b in range(Q):
                for l in range(N):
                    pred = ((c[0] if (a == k and b == l and Q > 1) else 0.0)
                            + (c[1] if (a == b and k == l) else 0.0)
                            + (c[2] if (a == l and k == b and Q > 1) else 0.0))
                    err = max(err, abs(pred - D[a * N + k, b * N + l]))
    scale = max(1.0, float(np.max(np.abs(D))) if D.size else 1.0)
    return c, err <= 1e-10 * scale


def _linear_in_fields(fn, names, what):
    """fn(theta) -> vector of values; returns (const part, {name: coeff
    vector}) assuming linearity in each named scalar datum, and checks it."""
    base = np.asarray(fn({}), dtype=float)
    coeffs = {}
    for nm in names:
        coeffs[nm] = np.asarray(fn({nm: 1.0}), dtype=float) - base
    rng = np.random.default_rng(1234)
    theta = {nm: float(rng.uniform(0.5, 2.0)) for nm in names}
    pred = base + sum(coeffs[nm] * theta[nm] for nm in names) if names else base
    got = np.asarray(fn(theta), dtype=float)
    if np.max(np.abs(pred - got), initial=0.0) > 1e-9 * max(1.0, np.max(np.abs(got), initial=0.0)):
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      f"{what} is not linear in the data fields")
    return base, coeffs


def _coef_terms(c_const, c_fields, fields):
    """Split a coefficient (const + sum of field * factor) into (coef dict)
    entries; each entry is one descriptor coefficient."""
    out = []
    if abs(c_const) > 0:
        out.append(_coef(L.COEF_CONST, 0, float(c_const)))
    for nm, v in c_fields.items():
        if abs(v) == 0:
            continue
        f = fields[nm]
        kind = L.COEF_ELEMENT if f.kind == "element" else L.COEF_NODAL
        out.append(_coef(kind, f.slot, float(v)))
    return out


def _lower_linear(tree, var, dim, fields, has_test2, probe=None):
    """Lower a weak form affine in u (or bilinear in Test/Test2)."""
    Q, N = var.qdim, dim
    P = probe(fields) if probe is not None else _Probe(tree, var, dim, fields)
    vals, grads = _basis(Q, N)
    zQ, zG = np.zeros(Q), np.zeros((Q, N))
    scal_fields = [nm for nm, f in fields.items() if f.kind in ("element", "nodal")]
    vec_fields = [nm for nm, f in fields.items() if f.kind == "vfield"]

    def trial(**kw):
        # the trial function is u (order-1 forms) or Test2_u (bilinear forms)
        if has_test2:
            return dict(U=zQ, GU=zG, V2=kw["U"], GV2=kw["GU"])
        return dict(U=kw["U"], GU=kw["GU"], V2=None, GV2=None)

    # coupling blocks as functions of theta
    def blocks(theta):
        out = []
        for V, GV in [(v, zG) for v in vals] + [(zQ, g) for g in grads]:
            base = P.eval(V=V, GV=GV, theta=theta, **trial(U=zQ, GU=zG))
            row = []
            for U, GU in [(v, zG) for v in vals] + [(zQ, g) for g in grads]:
                row.append(P.eval(V=V, GV=GV, theta=theta, **trial(U=U, GU=GU)) - base)
            out.append(row)
        return np.array(out)

    # affinity check in the trial function at a random state
    rng = np.random.default_rng(7)
    theta0 = {nm: float(rng.uniform(0.5, 2.0)) for nm in scal_fields}
    for nm in vec_fields:
        theta0[nm] = rng.uniform(-1, 1, fields[nm].qdim)
    Ur, GUr = rng.uniform(-1, 1, Q), rng.uniform(-1, 1, (Q, N))
    Vr, GVr = rng.uniform(-1, 1, Q), rng.uniform(-1, 1, (Q, N))
    B = blocks(theta0)
    lin = P.eval(V=Vr, GV=GVr, theta=theta0, **trial(U=Ur, GU=GUr))
    s0 = P.eval(V=Vr, GV=GVr, theta=theta0, **trial(U=zQ, GU=zG))
    vvec = np.concatenate([Vr, GVr.ravel()])
    uvec = np.concatenate([Ur, GUr.ravel()])
    pred = s0 + vvec @ B @ uvec
    if abs(pred - lin) > 1e-9 * max(1.0, abs(lin)):
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      "weak form is not affine in the variable")
    for nm in vec_fields:
        # vector fields may only enter the source part
        th = dict(theta0)
        th[nm] = th[nm] * 2.0
        if np.max(np.abs(blocks(th) - B)) > 1e-9 * max(1.0, np.max(np.abs(B))):
            if fields[nm].qdim == 1:
                # a scalar field on the variable's (scalar) mesh_fem that
                # multiplies the variable is a nodal coefficient
                f2 = dict(fields)
                f2[nm] = FieldInfo(nm, "nodal", 1, slot=fields[nm].slot)
                return _lower_linear(tree, var, dim, f2, has_test2, probe)
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          f"field {nm} multiplies the variable")

    # bilinear part: blocks linear in the scalar fields
    def flat_blocks(theta):
        th = dict(theta)
        for nm in vec_fields:
            th.setdefault(nm, np.zeros(fields[nm].qdim))
        return blocks(th).ravel()
    base, coeffs = _linear_in_fields(flat_blocks, scal_fields, "the bilinear coefficient")
    nQ = Q
    terms2 = []

    def split(Bflat):
        Bm = Bflat.reshape(Q + Q * N, Q + Q * N)
        vv, vg = Bm[:nQ, :nQ], Bm[:nQ, nQ:]
        gv, gg = Bm[nQ:, :nQ], Bm[nQ:, nQ:]
        tol = 1e-10 * max(1.0, np.max(np.abs(Bm)))
        if np.max(np.abs(vg), initial=0) > tol or np.max(np.abs(gv), initial=0) > tol:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          "value-gradient couplings are not lowered")
        cm = vv[0, 0]
        if np.max(np.abs(vv - cm * np.eye(Q)), initial=0) > tol:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "anisotropic mass term")
        c, ok = _iso_fit(gg, Q, N)
        if not ok:
            # a constant anisotropic coupling D[(a,k),(b,l)] (test (a,k),
            # trial (b,l)); K is symmetric only for a symmetric D
            if Q != 1 and Q != N:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                              "gradient coupling is not isotropic")
            if not np.array_equal(gg, gg.T):
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, "anisotropic gradient coupling is not symmetric")
            return cm, None, np.array(gg, dtype=float)
        return cm, c, None

    parts = [("", base)] + [(nm, coeffs[nm]) for nm in scal_fields]
    n_tensor = 0
    for nm, Bflat in parts:
        cm, c, Dt = split(Bflat)
        if Dt is not None:
            n_tensor += 1
            if n_tensor > 1:
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, "anisotropic couplings from more than one coefficient")
        if nm == "":
            if Dt is not None:
                t = _term(L.TERM_GRADGRAD_TENSOR, 1.0, [None, None, None])
                t["tensor"] = Dt.ravel().tolist()
                terms2.append(t)
            elif np.any(np.abs(c) > 0):
                terms2.append(_term(L.TERM_GRADGRAD, 1.0, [
                    _coef(L.COEF_CONST, 0, float(x)) if x != 0 else _coef(L.COEF_NONE)
                    for x in c]))
            if cm != 0:
                terms2.append(_term(L.TERM_MASS, 1.0, [_coef(L.COEF_CONST, 0, float(cm)), None, None]))
        else:
            f = fields[nm]
            kind = L.COEF_ELEMENT if f.kind == "element" else L.COEF_NODAL
            if Dt is not None:
                if kind != L.COEF_ELEMENT:
                    raise L.UnsupportedExpression(
                        L.E_UNSUPPORTED, "anisotropic coupling scaled by a nodal field")
                t = _term(L.TERM_GRADGRAD_TENSOR, 1.0, [_coef(kind, f.slot, 1.0), None, None])
                t["tensor"] = Dt.ravel().tolist()
                terms2.append(t)
            elif np.any(np.abs(c) > 0):
                terms2.append(_term(L.TERM_GRADGRAD, 1.0, [
                    _coef(kind, f.slot, float(x)) if x != 0 else _coef(L.COEF_NONE) for x in c]))
            if cm != 0:
                terms2.append(_term(L.TERM_MASS, 1.0, [_coef(kind, f.slot, float(cm)), None, None]))

    # source part (trial = 0): l(v) = sum_a s_a v_a (+ gradient sources rejected)
    terms1 = []
    if not has_test2:
        def src(theta):
            th = dict(theta)
            for nm in scal_fields:
                th.setdefault(nm, 1.0)
            out = []
            for V, GV in [(v, zG) for v in vals] + [(zQ, g) for g in grads]:
                out.append(P.eval(V=V, GV=GV, theta=th, U=zQ, GU=zG))
            return np.array(out)

        def src_of(nm_vec):
            def fn(theta):
                th = {}
                for nm in vec_fields:
                    th[nm] = np.zeros(fields[nm].qdim)
                if nm_vec is not None:
                    th[nm_vec] = theta.get("__x", np.zeros(fields[nm_vec].qdim))
                return src(th)
            return fn
        s_const = src_of(None)({})
        if np.max(np.abs(s_const)) > 0:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          "constant source terms are not lowered")
        for nm in vec_fields:
            f = fields[nm]
            fn = src_of(nm)
            cols = []
            for a in range(f.qdim):
                e = np.zeros(f.qdim)
                e[a] = 1.0
                cols.append(fn({"__x": e}))
            S = np.array(cols).T  # (Q + QN) x qdim_f
            if np.max(np.abs(S[Q:]), initial=0) > 0:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, "gradient source terms")
            if f.qdim != Q:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, "source field of wrong qdim")
            alpha = S[0, 0]
            if np.max(np.abs(S[:Q] - alpha * np.eye(Q))) > 1e-12 * max(1.0, abs(alpha)):
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, "anisotropic source")
            # the source must not depend on the scalar data fields
            for nm_s in scal_fields:
                def fn2(theta, nm_s=nm_s):
                    th = {nm2: np.zeros(fields[nm2].qdim) for nm2 in vec_fields}
                    th[nm] = np.ones(f.qdim)
                    th[nm_s] = theta.get("__s", 1.0)
                    out = []
                    for V, GV in [(v, zG) for v in vals] + [(zQ, g) for g in grads]:
                        out.append(P.eval(V=V, GV=GV, theta=th, U=zQ, GU=zG))
                    return np.array(out)
                if np.max(np.abs(fn2({"__s": 1.0}) - fn2({"__s": 3.0}))) > 0:
                    raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                                  "sources scaled by element data are not lowered")
            terms1.append(_term(L.TERM_SOURCE, float(alpha), [None, None, None],
                                field_slot=f.slot))
    return terms2, terms1


def _match_neohookean(tree, var):
    """((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[p1;p2]))):Grad_Test_u"""
    n = tree
    if n.kind != "bin" or n.value != ":":
        return None
    lhs, rhs = n.args
    if rhs.kind != "name" or rhs.value != "Grad_Test_" + var.name:
        return None
    if lhs.kind != "bin" or lhs.value != "*":
        return None
    F, S = lhs.args
    if not (F.kind == "bin" and F.value == "+"):
        return None
    idn, gu = F.args
    if not (idn.kind == "call" and idn.value == "Id" and gu.kind == "name"
            and gu.value == "Grad_" + var.name):
        return None
    if not (S.kind == "call" and S.value == "Compressible_Neo_Hookean_PK2" and len(S.args) == 2):
        return None
    a0, a1 = S.args
    if not (a0.kind == "name" and a0.value == "Grad_" + var.name):
        return None
    if a1.kind != "matrix" or len(a1.args) != 2 or any(len(r) != 1 for r in a1.args):
        return None
    return a1.args[0][0], a1.args[1][0]


def _match_neohookean_potential(tree, var):
    """Compressible_Neo_Hookean_potential(Grad_u,[p1;p2])"""
    S = tree
    if not (S.kind == "call" and S.value == "Compressible_Neo_Hookean_potential"
            and len(S.args) == 2):
        return None
    a0, a1 = S.args
    if not (a0.kind == "name" and a0.value == "Grad_" + var.name):
        return None
    if a1.kind != "matrix" or len(a1.args) != 2 or any(len(r) != 1 for r in a1.args):
        return None
    return a1.args[0][0], a1.args[1][0]


class _PolarProbe(_Probe):
    """Probe of a potential P(u) quadratic in (u, Grad_u): evaluates the
    polarisation (P(U + V) - P(U - V)) / 4 = B(U, V) + L(V) / 2, where
    P(u) = B(u, u) + L(u), as the affine weak form the linear lowering reads."""

    def eval(self, V=None, GV=None, theta=None, U=None, GU=None, V2=None, GV2=None):
        plus = float(evaluate(self.tree, self.env(U=U + V, GU=GU + GV, V=None, GV=None,
                                                  theta=theta)))
        minus = float(evaluate(self.tree, self.env(U=U - V, GU=GU - GV, V=None, GV=None,
                                                   theta=theta)))
        return (plus - minus) / 4.0


def _lower_potential(tree, var, dim, fields) -> "Lowered":
    """A potential quadratic in u: order 0 assembles P(u) = B(u,u) + L(u),
    order 1 its derivative 2 B(u, .) + L, order 2 the bilinear form 2 B (the
    derivatives GWFL's Diff gives for such a potential)."""
    Q, N = var.qdim, dim
    base = _Probe(tree, var, dim, fields)
    zQ, zG = np.zeros(Q), np.zeros((Q, N))
    th = {nm: 1.0 for nm, f in fields.items() if f.kind in ("element", "nodal")}
    for nm, f in fields.items():
        if f.kind == "vfield":
            th[nm] = np.ones(f.qdim)
    if abs(base.eval(U=zQ, GU=zG, V=None, GV=None, theta=th)) > 0:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      "potential terms independent of the variable")
    terms2, terms1 = _lower_linear(tree, var, dim, fields, False,
                                   probe=lambda f: _PolarProbe(tree, var, dim, f))
    if any(t["kind"] == L.TERM_GRADGRAD_TENSOR for t in terms2):
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      "anisotropic couplings in potentials are not lowered")
    # quadratic check: P(2u) = 4 B(u,u) + 2 L(u)
    rng = np.random.default_rng(99)
    Ur, GUr = rng.uniform(-1, 1, Q), rng.uniform(-1, 1, (Q, N))
    p1 = base.eval(U=Ur, GU=GUr, V=None, GV=None, theta=th)
    p2 = base.eval(U=2 * Ur, GU=2 * GUr, V=None, GV=None, theta=th)
    pm = base.eval(U=-Ur, GU=-GUr, V=None, GV=None, theta=th)
    quad, lin = (p1 + pm) / 2.0, (p1 - pm) / 2.0
    if abs(p2 - (4 * quad + 2 * lin)) > 1e-9 * max(1.0, abs(p2)):
        raise L.UnsupportedExpression(L.E_UNSUPPORTED, "potential is not quadratic in u")
    src = []
    for t in terms1:
        t2 = dict(t)
        t2["scale"] = 2.0 * t["scale"]   # the probe saw L / 2
        src.append(t2)
    dbl = []
    for t in terms2:
        t2 = dict(t)
        t2["scale"] = 2.0 * t["scale"]
        dbl.append(t2)
    return Lowered(order2=dbl, order1=dbl + src, order0=terms2 + src, max_order=0)


def _internal_pressure_part(tree, var, dim, fields, pname):
    """u equation of a displacement / pressure pair: the part of the weak form
    that the internal variable p contributes must be sp p Div_Test_u, with sp
    a constant (the reference's (-p*Id(meshdim)):Grad_Test_u has sp = -1)."""
    Q, N = var.qdim, dim
    P = _Probe(tree, var, dim, fields)
    vals, grads = _basis(Q, N)
    zQ, zG = np.zeros(Q), np.zeros((Q, N))
    th0 = {nm: 1.0 for nm, f in fields.items() if f.kind in ("element", "nodal")}
    rng = np.random.default_rng(11)
    Ur, GUr = rng.uniform(-1, 1, Q), rng.uniform(-1, 1, (Q, N))
    sp = None
    for V, GV in [(v, zG) for v in vals] + [(zQ, g) for g in grads]:
        for th_extra in ({}, {nm: 2.0 for nm in th0}):
            th = dict(th0, **th_extra)
            d1 = P.eval(V=V, GV=GV, theta=dict(th, **{pname: 1.0}), U=zQ, GU=zG) - \
                P.eval(V=V, GV=GV, theta=th, U=zQ, GU=zG)
            d2 = P.eval(V=V, GV=GV, theta=dict(th, **{pname: 2.0}), U=Ur, GU=GUr) - \
                P.eval(V=V, GV=GV, theta=th, U=Ur, GU=GUr)
            div = float(np.trace(GV)) if Q == N and Q > 1 else 0.0
            if sp is None and div != 0.0:
                sp = d1 / div
            want1 = (sp or 0.0) * div
            if abs(d1 - want1) > 1e-12 * max(1.0, abs(d1)) or \
                    abs(d2 - 2.0 * want1) > 1e-12 * max(1.0, abs(d2)):
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, f"the internal variable {pname} must enter the "
                    f"displacement equation as (c {pname} Id(meshdim)):Grad_Test_u")
    if not sp:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"{pname} does not couple to Test_u")
    return float(sp)


def _internal_equation(tree, var, dim, fields, pname):
    """p equation: the weak form times Test_p must be
    scale (p + c3 p^3 + kb Div_u), kb a constant or one element / nodal datum
    times a constant, scale and c3 constants."""
    Q, N = var.qdim, dim
    if Q != N or Q != 3:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      "internal pressure equations on 3-D vector fields only")
    scal = [nm for nm, f in fields.items() if f.kind in ("element", "nodal")]
    zQ, zG = np.zeros(Q), np.zeros((Q, N))

    def f(p, GU, theta=None, U=None):
        th = dict(theta or {})
        th[pname] = p
        env = _Probe(tree, var, dim, fields).env(U=zQ if U is None else U, GU=GU, V=None,
                                                  GV=None, theta=th)
        env["Test_" + pname] = 1.0
        return float(evaluate(tree, env))
    th1 = {nm: 1.0 for nm in scal}
    if abs(f(0.0, zG, th1)) > 0:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      f"constant terms in the {pname} equation are not lowered")
    s1, s2 = f(1.0, zG, th1), f(2.0, zG, th1)
    scale = (8.0 * s1 - s2) / 6.0
    c3s = (s2 - 2.0 * s1) / 6.0
    if scale == 0.0:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"{pname} equation without a {pname} term")
    for pv in (0.7, -1.3):
        want = scale * pv + c3s * pv ** 3
        for th in (th1, {nm: 2.5 for nm in scal}):
            if abs(f(pv, zG, th) - want) > 1e-12 * max(1.0, abs(want)):
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, f"the {pname} equation must be scale ({pname} + "
                    f"c {pname}^3 + k Div_u) with constant scale and c")

    # the Div_u coefficient, linear in the scalar data fields
    def kb_of(theta):
        return np.array([f(0.0, np.diag([1.0, 0.0, 0.0]), theta)])
    base, coeffs = _linear_in_fields(kb_of, scal, f"the Div_{var.name} coefficient")
    entries = _coef_terms(base[0] / scale, {k: v[0] / scale for k, v in coeffs.items()}, fields)
    if len(entries) != 1:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      f"the Div_{var.name} coefficient must be one field "
                                      "times a constant")
    # isotropy (a multiple of Div_u) and no other dependence on u or cross terms
    rng = np.random.default_rng(5)
    th = {nm: float(rng.uniform(0.5, 2.0)) for nm in scal}
    kb = float(kb_of(th)[0])
    GUr, Ur = rng.uniform(-1, 1, (Q, N)), rng.uniform(-1, 1, Q)
    for pv in (0.0, 0.9):
        want = scale * pv + c3s * pv ** 3 + kb * float(np.trace(GUr))
        if abs(f(pv, GUr, th, Ur) - want) > 1e-10 * max(1.0, abs(want)):
            raise L.UnsupportedExpression(
                L.E_UNSUPPORTED, f"the {pname} equation depends on {var.name} other than "
                f"through Div_{var.name}")
    c3 = c3s / scale
    return {"name": pname, "scale": float(scale),
            "c3": _coef(L.COEF_CONST, 0, float(c3)) if c3 != 0 else None,
            "kb": entries[0]}


def lower(expr: str, var: FieldInfo, dim: int, fields: dict, add_derivative_order=2) -> Lowered:
    """Lower a GWFL expression over one fem variable to descriptor terms."""
    tree = parse(expr)
    used = names_in(tree)
    name = var.name
    has_test = any(s in used for s in ("Test_" + name, "Grad_Test_" + name, "Div_Test_" + name))
    has_test2 = any(s in used for s in ("Test2_" + name, "Grad_Test2_" + name, "Div_Test2_" + name))
    for s in used:
        if s.endswith("()"):
            continue
        base = s
        for pre in ("Grad_Test2_", "Div_Test2_", "Test2_", "Grad_Test_", "Div_Test_", "Test_",
                    "Grad_", "Div_"):
            if s.startswith(pre):
                base = s[len(pre):]
                break
        if base in ("meshdim", "pi", "qdim"):
            continue
        if base != name and base not in fields:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"unknown name {s!r} in {expr!r}")
        if base != name and s != base and not (
                fields[base].kind == "internal" and s == "Test_" + base):
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          f"derivatives of data fields ({s}) are not lowered")
    if has_test2 and not has_test:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED, "Test2 without Test")
    internal = [nm for nm, f in fields.items() if f.kind == "internal"]
    for pname in internal:
        if any(s in used for s in ("Grad_" + pname, "Test2_" + pname, "Grad_Test_" + pname)):
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          f"{pname} is an im_data variable: no gradient")
        if "Test_" + pname in used:
            if has_test or has_test2:
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, f"Test_{pname} and Test_{name} in one expression")
            part = _internal_equation(tree, var, dim, fields, pname)
            return Lowered(order2=[], order1=[], order0=[], max_order=2, internal=part)
    used_int = [nm for nm in internal if nm in used]
    if used_int:
        if len(used_int) > 1 or not has_test or has_test2:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                          "one internal variable, in a residual-form term")
        pname = used_int[0]
        sp = _internal_pressure_part(tree, var, dim, fields, pname)
        # the rest of the expression, with p = 0 (the probe's default)
        terms2, terms1 = _lower_linear(tree, var, dim, fields, False)
        return Lowered(order2=terms2, order1=terms2 + terms1, order0=[], max_order=2,
                       internal={"name": pname, "sp": sp})
    nh = _match_neohookean(tree, var)
    nh_pot = None if has_test else _match_neohookean_potential(tree, var)
    if not has_test and nh_pot is None:
        return _lower_potential(tree, var, dim, fields)
    if nh is not None or nh_pot is not None:
        nh = nh if nh is not None else nh_pot
        if dim != 3 or var.qdim != 3:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "neo-Hookean law is 3-D only")
        coefs = []
        scal = [nm for nm, f in fields.items() if f.kind in ("element", "nodal")]
        for p in nh:
            def fn(theta, p=p):
                env = {"meshdim": float(dim), "pi": math.pi}
                for f in fields.values():
                    if f.kind == "const":
                        env[f.name] = f.value
                    elif f.kind in ("element", "nodal"):
                        env[f.name] = theta.get(f.name, 0.0)
                return np.array([float(evaluate(p, env))])
            c0, cf = _linear_in_fields(fn, scal, "a hyperelastic parameter")
            entries = _coef_terms(c0[0], {k: v[0] for k, v in cf.items()}, fields)
            if len(entries) > 1:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                              "a law parameter must be one field times a constant")
            coefs.append(entries[0] if entries else _coef(L.COEF_CONST, 0, 0.0))
        t = _term(L.TERM_NEOHOOKEAN, 1.0, [coefs[0], coefs[1], None])
        if nh_pot is not None:
            # the potential, and its first and second derivatives in u (the
            # PK2 residual and tangent)
            return Lowered(order2=[t], order1=[t], order0=[t], max_order=0)
        return Lowered(order2=[t], order1=[t], order0=[], max_order=2)
    terms2, terms1 = _lower_linear(tree, var, dim, fields, has_test2)
    if has_test2:
        return Lowered(order2=terms2, order1=[], order0=[], max_order=2)
    return Lowered(order2=terms2 if add_derivative_order >= 2 else [],
                   order1=terms2 + terms1, order0=[], max_order=2 if add_derivative_order >= 2 else 1)


def to_form(terms: list) -> L.Form:
    f = L.Form()
    if len(terms) > L.MAX_TERMS:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED, "too many terms")
    if sum(t["kind"] == L.TERM_GRADGRAD_TENSOR for t in terms) > 1:
        raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                      "more than one anisotropic gradient coupling in one form")
    f.n_terms = len(terms)
    for i, t in enumerate(terms):
        T = f.terms[i]
        T.kind = t["kind"]
        T.scale = t["scale"]
        T.field_slot = t["field_slot"]
        T.aux_slot = t.get("aux_slot", 0)
        for k in range(3):
            c = t["c"][k]
            if c is None:
                T.c[k].kind = L.COEF_NONE
                T.c[k].slot = 0
                T.c[k].value = 0.0
            else:
                T.c[k].kind = c["kind"]
                T.c[k].slot = c["slot"]
                T.c[k].value = c["value"]
        if t.get("tensor") is not None:
            for k, x in enumerate(t["tensor"]):
                f.tensor[k] = float(x)
    return f
