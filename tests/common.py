"""Shared helpers of the test-suite: fixtures of the reference, problem
construction for the oracle and the GPU path, and CSR comparison."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

import getfem_gb300 as g
from getfem_gb300 import _lib as L
from getfem_gb300 import gwfl

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# value tolerance: |a - b| <= RTOL * max(|b|, FLOOR * max|row of b|)
RTOL = 1e-12
FLOOR = 1e-3


def golden_names(condensed=False):
    """Fixture names: the plain assembly cases, or (condensed=True) the
    internal-variable condensation cases (they carry R_full / Rc)."""
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        with np.load(p) as z:
            if ("Rc" in z.files) == condensed:
                out.append(os.path.basename(p)[:-4])
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    rec = {k: z[k] for k in z.files}
    rec["meta"] = json.loads(str(rec["meta"]))
    return rec


def build_case(rec):
    """Mesh, MeshFem, MeshIm and a populated GaWorkspace for a fixture."""
    m = rec["meta"]
    kind = "simplex" if m["gt"] == "PK" else "hex"
    mesh = g.Mesh.regular_unit(m["dim"], m["nx"], kind, jitter=rec.get("jitter"))
    mf = g.MeshFem(mesh, m["qdim"], degree=m["degree"])
    mim = g.MeshIm(mesh, m["im"])
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rec["in_u"])
    mf0 = None
    for cname, ck in m["consts"].items():
        v = rec["in_" + cname]
        if ck == "P0":
            mf0 = mf0 or g.MeshFem(mesh, 1, degree=0)
            ws.add_fem_constant(cname, mf0, v)
        elif ck == "V":
            ws.add_fem_constant(cname, mf, v)
        elif ck == "S":
            ws.add_fem_constant(cname, g.MeshFem(mesh, 1, degree=m["degree"]), v)
        elif ck == "C":
            ws.add_fixed_size_constant(cname, v)
    ws.add_expression(m["expr"], mim)
    return mesh, mf, mim, ws


def slots_of(ws):
    return {d.slot: np.asarray(d.values, dtype=float) for d in ws.data.values() if d.slot >= 0}


def oracle_problem(mesh, mf, mim, terms, slots):
    from oracle import gfref
    return gfref.Problem(mesh.dim, mesh.kind, mf.degree, mf.qdim, mim.im, mesh.points,
                         mesh.cvpts, mf.dofs, mf.nb_dof(), terms, slots)


def golden_csr(rec):
    import scipy.sparse as sp
    n = rec["meta"]["n_dof"]
    return sp.csr_matrix((rec["K_vals"], rec["K_colidx"], rec["K_rowptr"]), shape=(n, n))


def assert_same_pattern(A, B):
    A = A.tocsr()
    B = B.tocsr()
    assert A.shape == B.shape
    assert np.array_equal(np.asarray(A.indptr, dtype=np.int64), np.asarray(B.indptr, dtype=np.int64)), \
        "row pointers differ"
    assert np.array_equal(np.asarray(A.indices, dtype=np.int64), np.asarray(B.indices, dtype=np.int64)), \
        "column indices differ"


def value_errors(A, B):
    """Entry-wise errors of A against the reference B (same pattern), scaled
    by max(|b|, FLOOR * max|row of B|)."""
    B = B.tocsr()
    a = np.asarray(A.tocsr().data)
    b = np.asarray(B.data)
    rows = np.repeat(np.arange(B.shape[0]), np.diff(B.indptr))
    rmax = np.zeros(B.shape[0])
    np.maximum.at(rmax, rows, np.abs(b))
    scale = np.maximum(np.abs(b), FLOOR * rmax[rows])
    scale[scale == 0] = 1.0
    return np.abs(a - b) / scale


def vec_errors(a, b):
    scale = np.maximum(np.abs(b), FLOOR * np.max(np.abs(b)))
    scale[scale == 0] = 1.0
    return np.abs(a - b) / scale


def build_condensed_case(rec):
    """Mesh, MeshFem, MeshIm and a GaWorkspace holding u, the internal
    variable p and both expressions of a condensation fixture."""
    m = rec["meta"]
    kind = "simplex" if m["gt"] == "PK" else "hex"
    mesh = g.Mesh.regular_unit(m["dim"], m["nx"], kind, jitter=rec.get("jitter"))
    mf = g.MeshFem(mesh, m["qdim"], degree=m["degree"])
    mim = g.MeshIm(mesh, m["im"])
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rec["in_u"])
    ws.add_internal_im_variable("p", g.ImData(mim), rec["in_p"])
    for cname, ck in m["consts"].items():
        v = rec["in_" + cname]
        if ck == "P0":
            ws.add_fem_constant(cname, g.MeshFem(mesh, 1, degree=0), v)
        else:
            ws.add_fixed_size_constant(cname, v)
    ws.add_expression(m["expr"], mim)
    ws.add_expression(m["expr2"], mim)
    return mesh, mf, mim, ws


def csr_errors(A, B):
    """Errors of A against the reference B on the union of their patterns,
    scaled by max(|b|, FLOOR * max|row of B|): entries one side stores and
    the other drops must be below the floor."""
    import scipy.sparse as sp
    A = sp.csr_matrix(A)
    B = sp.csr_matrix(B)
    D = (A - B).tocoo()
    rmax = np.asarray(abs(B).max(axis=1).todense()).ravel()
    b = np.asarray(B[D.row, D.col]).ravel()
    scale = np.maximum(np.abs(b), FLOOR * rmax[D.row])
    scale[scale == 0] = 1.0
    return np.abs(D.data) / scale if D.nnz else np.zeros(1)
