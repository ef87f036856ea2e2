"""ORACLE — test infrastructure only.

ctypes loader of oracle/_build/libgfref.so, the CPU restatement of GetFEM's
generic-assembly hot path (oracle/gfref.cc).  Imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, as the checker;
the getfem_gb300 package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from math import comb

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libgfref.so")
MAX_SLOTS = 8


def build() -> str:
    src = [os.path.join(HERE, f) for f in ("gfref.cc", "gfref.h", "Makefile")]
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["make", "-C", HERE], check=True, capture_output=True)
    return LIB


class _Coef(C.Structure):
    _fields_ = [("kind", C.c_int32), ("slot", C.c_int32), ("value", C.c_double)]


class _Term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("field_slot", C.c_int32), ("scale", C.c_double),
                ("c", _Coef * 3), ("aux_slot", C.c_int32), ("reserved", C.c_int32)]


class _Form(C.Structure):
    _fields_ = [("n_terms", C.c_int32), ("terms", _Term * 8), ("tensor", C.c_double * 81)]


class _Problem(C.Structure):
    _fields_ = [("dim", C.c_int32), ("kind", C.c_int32), ("degree", C.c_int32),
                ("qdim", C.c_int32), ("im", C.c_char_p), ("n_points", C.c_int64),
                ("n_elements", C.c_int64), ("n_dof", C.c_int64),
                ("points", C.c_void_p), ("cvpts", C.c_void_p), ("dofs", C.c_void_p),
                ("form", _Form), ("slots", C.c_void_p * MAX_SLOTS)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.gfref_assemble_matrix.restype = C.c_void_p
        L.gfref_assemble_matrix.argtypes = [C.POINTER(_Problem), C.c_int, C.POINTER(C.c_int64)]
        L.gfref_matrix_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.gfref_matrix_free.argtypes = [C.c_void_p]
        L.gfref_assemble_vector.argtypes = [C.POINTER(_Problem), C.c_int, C.c_void_p]
        L.gfref_assemble_potential.argtypes = [C.POINTER(_Problem), C.c_int, C.POINTER(C.c_double)]
        L.gfref_assemble_vector_internal.argtypes = [C.POINTER(_Problem), C.c_int, C.c_void_p,
                                                     C.c_void_p]
        L.gfref_assemble_condensed.restype = C.c_void_p
        L.gfref_assemble_condensed.argtypes = [C.POINTER(_Problem), C.c_int,
                                               C.POINTER(C.c_int64), C.c_void_p, C.c_void_p,
                                               C.c_void_p]
        L.gfref_tables.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, C.POINTER(C.c_int),
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Problem:
    """One discretisation + lowered form + data, as the oracle sees it.

    terms: list of term dicts as produced by getfem_gb300.gwfl (kind, scale,
    field_slot, c=[coef dicts or None]); slots: {slot: numpy array}."""

    def __init__(self, dim, kind, degree, qdim, im, points, cvpts, dofs, n_dof, terms, slots):
        self._keep = []
        P = _Problem()
        P.dim, P.kind, P.degree, P.qdim = dim, kind, degree, qdim
        self._im = im.encode()
        P.im = self._im
        pts = np.ascontiguousarray(points, dtype=np.float64)
        cv = np.ascontiguousarray(cvpts, dtype=np.int64)
        dd = np.ascontiguousarray(dofs, dtype=np.int64)
        self._keep += [pts, cv, dd]
        P.n_points, P.n_elements, P.n_dof = pts.shape[0], cv.shape[0], n_dof
        P.points, P.cvpts, P.dofs = _p(pts), _p(cv), _p(dd)
        P.form.n_terms = len(terms)
        for i, t in enumerate(terms):
            T = P.form.terms[i]
            T.kind, T.scale, T.field_slot = t["kind"], t["scale"], t["field_slot"]
            T.aux_slot = t.get("aux_slot", 0)
            for k in range(3):
                c = t["c"][k]
                if c is not None:
                    T.c[k].kind, T.c[k].slot, T.c[k].value = c["kind"], c["slot"], c["value"]
            if t.get("tensor") is not None:
                for k, x in enumerate(t["tensor"]):
                    P.form.tensor[k] = float(x)
        for s, v in slots.items():
            a = np.ascontiguousarray(v, dtype=np.float64)
            self._keep.append(a)
            P.slots[s] = _p(a).value
        self.P = P
        self.n_dof = n_dof
        nb = comb(degree + dim, dim) if kind == 0 else (degree + 1) ** dim
        self.row_len = nb * qdim

    def matrix(self, nthreads: int = 1):
        import scipy.sparse as sp
        nnz = C.c_int64()
        h = lib().gfref_assemble_matrix(C.byref(self.P), nthreads, C.byref(nnz))
        if not h:
            raise RuntimeError("oracle assembly failed")
        rowptr = np.empty(self.n_dof + 1, dtype=np.int64)
        colidx = np.empty(nnz.value, dtype=np.int64)
        vals = np.empty(nnz.value)
        lib().gfref_matrix_copy(h, _p(rowptr), _p(colidx), _p(vals))
        lib().gfref_matrix_free(h)
        return sp.csr_matrix((vals, colidx, rowptr), shape=(self.n_dof, self.n_dof))

    def vector(self, nthreads: int = 1):
        V = np.zeros(self.n_dof)
        if lib().gfref_assemble_vector(C.byref(self.P), nthreads, _p(V)) != 0:
            raise RuntimeError("oracle assembly failed")
        return V

    def _n_internal(self):
        nq = C.c_int()
        lib().gfref_tables(self.P.dim, self.P.kind, self.P.degree, self.P.im, C.byref(nq),
                           None, None, None, None)
        return self.P.n_elements * nq.value, nq.value

    def vector_internal(self, nthreads: int = 1):
        """Order 1 of a form with an internal variable: (V, internal residual)."""
        V = np.zeros(self.n_dof)
        Vint = np.zeros(self._n_internal()[0])
        if lib().gfref_assemble_vector_internal(C.byref(self.P), nthreads, _p(V), _p(Vint)) != 0:
            raise RuntimeError("oracle assembly failed")
        return V, Vint

    def condensed(self, nthreads: int = 1):
        """Order 2 with static condensation of the internal variable (its
        cached residual in the term's aux slot): (K, V, RQpr, KQJpr rows)."""
        import scipy.sparse as sp
        n_int, _ = self._n_internal()
        s = self.row_len
        V = np.zeros(self.n_dof)
        Vint = np.zeros(n_int)
        cpl = np.zeros(n_int * s)
        nnz = C.c_int64()
        h = lib().gfref_assemble_condensed(C.byref(self.P), nthreads, C.byref(nnz), _p(V),
                                           _p(Vint), _p(cpl))
        if not h:
            raise RuntimeError("oracle assembly failed")
        rowptr = np.empty(self.n_dof + 1, dtype=np.int64)
        colidx = np.empty(nnz.value, dtype=np.int64)
        vals = np.empty(nnz.value)
        lib().gfref_matrix_copy(h, _p(rowptr), _p(colidx), _p(vals))
        lib().gfref_matrix_free(h)
        K = sp.csr_matrix((vals, colidx, rowptr), shape=(self.n_dof, self.n_dof))
        return K, V, Vint, cpl.reshape(n_int, s)

    def potential(self, nthreads: int = 1):
        E = C.c_double()
        if lib().gfref_assemble_potential(C.byref(self.P), nthreads, C.byref(E)) != 0:
            raise RuntimeError("oracle assembly failed")
        return E.value


def tables(dim, kind, degree, im):
    nq = C.c_int()
    lib().gfref_tables(dim, kind, degree, im.encode(), C.byref(nq), None, None, None, None)
    nb = {0: None}
    # number of basis functions
    if kind == 0:
        from math import comb
        n = comb(degree + dim, dim)
    else:
        n = (degree + 1) ** dim
    pts = np.empty((nq.value, dim))
    w = np.empty(nq.value)
    val = np.empty((nq.value, n))
    grad = np.empty((nq.value, n, dim))
    lib().gfref_tables(dim, kind, degree, im.encode(), C.byref(nq), _p(pts), _p(w), _p(val), _p(grad))
    del nb
    return pts, w, val, grad
