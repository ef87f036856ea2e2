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
        if os.path.basename(p).startswith("full_") or p.endswith("_diff.npz"):
            continue  # full-size records (test_fullsize.py), parameter gradients
            # (test_adjoint_diff.py)
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


# ------------------------------------------------ full-size fixtures
# (tests/golden/full_*.npz, made by tests/golden/make_fullsize.py from the
# reference on the benchmark workloads' own inputs)

def sha256_i64(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def _row_max(indptr, data):
    """max |entry| of every row (rows may be empty)."""
    n = indptr.size - 1
    out = np.zeros(n)
    nonempty = np.flatnonzero(np.diff(indptr) > 0)
    if nonempty.size:
        out[nonempty] = np.maximum.reduceat(np.abs(data), indptr[nonempty])
    return out


def fullsize_report(rec, indptr, indices, data, R, probes=True):
    """Compares an assembled K (CSR arrays) and R with a full-size fixture.
    Returns a dict of the checks: pattern hashes and nnz (bit-exact), the
    scaled errors of the kept rows, single entries and R values, and the
    bilinear probes' errors relative to their absolute sums."""
    indptr = np.asarray(indptr, dtype=np.int64)
    indices = np.asarray(indices)
    data = np.asarray(data)
    R = np.asarray(R)
    out = {"nnz": int(indptr[-1]) == int(rec["nnz"][0]),
           "rowptr": sha256_i64(indptr) == str(rec["rowptr_sha256"]),
           "colidx": sha256_i64(indices) == str(rec["colidx_sha256"])}
    rmax = _row_max(indptr, data)
    if "K_vals" in rec:  # kept whole
        import scipy.sparse as sp
        n = indptr.size - 1
        A = sp.csr_matrix((data, indices, indptr), shape=(n, n))
        B = sp.csr_matrix((rec["K_vals"], rec["K_colidx"], rec["K_rowptr"]), shape=(n, n))
        out["K_err"] = float(value_errors(A, B).max())
        out["R_err"] = float(vec_errors(R, rec["R"]).max())
    else:
        errs, same_cols = [], True
        rows, rptr = rec["rows"], rec["rows_ptr"]
        for k, r in enumerate(rows):
            a0, a1 = indptr[r], indptr[r + 1]
            cols_ref = rec["rows_col"][rptr[k]:rptr[k + 1]]
            vals_ref = rec["rows_val"][rptr[k]:rptr[k + 1]]
            if a1 - a0 != cols_ref.size or not np.array_equal(indices[a0:a1], cols_ref):
                same_cols = False
                continue
            scale = np.maximum(np.abs(vals_ref), FLOOR * np.abs(vals_ref).max())
            scale[scale == 0] = 1.0
            errs.append((np.abs(data[a0:a1] - vals_ref) / scale).max())
        out["rows_cols"] = same_cols
        ent_err, found = [], True
        for r, c, v in zip(rec["ent_row"], rec["ent_col"], rec["ent_val"]):
            a0, a1 = indptr[r], indptr[r + 1]
            p = a0 + np.searchsorted(indices[a0:a1], c)
            if p >= a1 or indices[p] != c:
                found = False
                continue
            ent_err.append(abs(data[p] - v) / max(abs(v), FLOOR * rmax[r], 1e-300))
        out["entries_found"] = found
        out["K_err"] = float(max(errs + ent_err)) if errs or ent_err else float("inf")
        rv = rec["R_val"]
        scale = np.maximum(np.abs(rv), FLOOR * float(rec["R_max"][0]))
        scale[scale == 0] = 1.0
        out["R_err"] = float((np.abs(R[rec["R_idx"]] - rv) / scale).max())
    if probes:
        n = indptr.size - 1
        rng = np.random.default_rng(int(rec["meta"]["probe_seed"]))
        row_of = np.repeat(np.arange(n), np.diff(indptr))
        pk, pr = [], []
        for k in range(rec["probe_wKv"].size):
            w, v = rng.standard_normal(n), rng.standard_normal(n)
            t = w[row_of] * data * v[indices]
            pk.append(abs(t.sum() - rec["probe_wKv"][k]) / rec["probe_wKv_abs"][k])
            pr.append(abs(w @ R - rec["probe_wR"][k]) / rec["probe_wR_abs"][k])
        out["probe_K_err"] = float(max(pk))
        out["probe_R_err"] = float(max(pr))
    return out


def assert_fullsize(rep):
    """The bar of the full-size comparison: pattern bit-exact, values within
    RTOL (scaled as everywhere), probes within 2*RTOL of their absolute sums
    (their own summation rounding stays below 1e-14 of it)."""
    for k in ("nnz", "rowptr", "colidx", "rows_cols", "entries_found"):
        assert rep.get(k, True), (k, rep)
    assert rep["K_err"] <= RTOL, rep
    assert rep["R_err"] <= RTOL, rep
    if "probe_K_err" in rep:
        assert rep["probe_K_err"] <= 2 * RTOL, rep
        assert rep["probe_R_err"] <= 2 * RTOL, rep
