"""GaWorkspace: the ga_workspace interface of GetFEM on the GPU backend.

Mirrors getfem::ga_workspace (getfem/getfem_generic_assembly.h:378-600):
add_fem_variable / add_fem_constant / add_fixed_size_constant,
add_expression(expr, mim, region, add_derivative_order) and
assembly(order), with assembled_matrix / assembled_vector getters and the
set_assembled_matrix / set_assembled_vector setters whose targets are
accumulated into, as the reference accumulates into an external K
(src/getfem_generic_assembly_workspace.cc:803-845).

Internal im_data variables (add_internal_im_variable: a pressure p per
element Gauss point in a displacement / pressure pair) are condensed out by
assembly(order, condensation=True) as ga_workspace::assembly(order, true)
does (getfem_generic_assembly_compile_and_exec.cc:5562-5790, :8429-8640):
order 1 gives [R_u; R_p], order 2 the condensed K, the vector
[-K_up K_pp^-1 R_p; K_pp^-1 R_p / (w J)] and internal_coupling_matrix()
(K_pp^-1 K_pu), reading R_p from the assembled vector.

Expressions are lowered when added (gwfl.lower); unsupported ones raise
UnsupportedExpression there, as ga_compile would reject them.  Assembly
runs on the GPU through the C ABI (one plan per variable, integration
method and form); results are returned as scipy CSR / numpy on the host, or
left on the device (assembled_matrix_device).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import gwfl
from .mesh import MeshFem, MeshIm


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


class _Datum:
    def __init__(self, name, kind, mf=None, values=None, slot=-1):
        self.name = name
        self.kind = kind        # 'variable', 'fem_constant', 'fixed', 'internal',
                                # 'internal_res' (the residual condensation reads)
        self.mf = mf
        self.values = values
        self.slot = slot


class _Group:
    """Expressions over one variable and one integration method."""

    def __init__(self, var: _Datum, mim: MeshIm):
        self.var = var
        self.mim = mim
        self.order2 = []
        self.order1 = []
        self.order0 = []
        self.internal = {}  # parts of a displacement / internal pressure pair
        self.plans = {}   # key: tuple(form terms) -> plan handle

    def internal_term(self, ws):
        """The TERM_INTERNAL_P of the group (None without internal variable)."""
        if not self.internal:
            return None
        I = self.internal
        if "sp" not in I or "scale" not in I:
            raise L.UnsupportedExpression(
                L.E_UNSUPPORTED, f"internal variable {I['name']}: both the displacement "
                "and the internal equation are needed")
        d = ws.data[I["name"]]
        r = ws.data[I["name"] + "#res"]
        return {"kind": L.TERM_INTERNAL_P, "scale": I["scale"], "field_slot": d.slot,
                "aux_slot": r.slot,
                "c": [gwfl._coef(L.COEF_CONST, 0, I["sp"]), I["kb"], I["c3"]]}


def _terms_key(terms):
    out = []
    for t in terms:
        cs = tuple(None if c is None else (c["kind"], c["slot"], c["value"]) for c in t["c"])
        out.append((t["kind"], t["scale"], t["field_slot"], t.get("aux_slot", 0), cs))
    return tuple(out)


class GaWorkspace:
    def __init__(self, stream=None):
        self.data = {}
        self.groups = []
        self._K = None
        self._V = None
        self._E = None
        self._ext_K = None
        self._ext_V = None
        self._KQJ = None
        self._ext_KQJ = None
        self._slots = 1  # slot 0 is the variable
        self._stream = stream
        self._plans = []

    # ----------------------------------------------------------- variables
    def add_fem_variable(self, name: str, mf: MeshFem, I=None, U=None):
        if any(d.kind == "variable" for d in self.data.values()):
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "one fem variable per workspace")
        if U is None:
            U = np.zeros(mf.nb_dof())
        self.data[name] = _Datum(name, "variable", mf, U, L.SLOT_U)

    def add_fem_constant(self, name: str, mf: MeshFem, V):
        self._new_slot(name, _Datum(name, "fem_constant", mf, V))

    def add_fixed_size_constant(self, name: str, V):
        self.data[name] = _Datum(name, "fixed", None, np.atleast_1d(np.asarray(V, dtype=float)))

    def add_internal_im_variable(self, name: str, imd, VV=None):
        """An internal variable on im_data points (condensed at assembly),
        ga_workspace::add_internal_im_variable (getfem_generic_assembly.h:459).
        VV: n_elements * nq values (numpy or a CUDA tensor)."""
        if imd.nb_tensor_elem() != 1:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "scalar internal variables only")
        if any(d.kind == "internal" for d in self.data.values()):
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "one internal variable per workspace")
        if VV is None:
            VV = np.zeros(imd.nb_index())
        d = _Datum(name, "internal", None, VV)
        d.imd = imd
        self._new_slot(name, d)
        self._new_slot(name + "#res", _Datum(name + "#res", "internal_res"))

    def is_internal_variable(self, name: str) -> bool:
        return name in self.data and self.data[name].kind == "internal"

    def nb_internal_dof(self) -> int:
        return sum(d.imd.nb_index() for d in self.data.values() if d.kind == "internal")

    def set_variable_value(self, name: str, U):
        self.data[name].values = U

    def _new_slot(self, name, d):
        if name in self.data:
            d.slot = self.data[name].slot
        else:
            if self._slots >= L.MAX_SLOTS:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, "too many data fields")
            d.slot = self._slots
            self._slots += 1
        self.data[name] = d

    # --------------------------------------------------------- expressions
    def _field_infos(self, var: _Datum):
        out = {}
        vmf = var.mf
        for d in self.data.values():
            if d.kind in ("variable", "internal_res"):
                continue
            if d.kind == "internal":
                if d.imd.mim.mesh is not vmf.mesh:
                    raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"{d.name} is on another mesh")
                out[d.name] = gwfl.FieldInfo(d.name, "internal", 1, slot=d.slot)
                continue
            if d.kind == "fixed":
                v = d.values
                out[d.name] = gwfl.FieldInfo(d.name, "const", value=float(v[0]) if v.size == 1 else v)
                continue
            mf = d.mf
            if mf.mesh is not vmf.mesh:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"{d.name} is on another mesh")
            if mf.degree == 0 and mf.qdim == 1:
                out[d.name] = gwfl.FieldInfo(d.name, "element", 1, slot=d.slot)
            elif mf.degree == vmf.degree and mf.qdim == vmf.qdim:
                out[d.name] = gwfl.FieldInfo(d.name, "vfield", mf.qdim, slot=d.slot)
            elif mf.degree == vmf.degree and mf.qdim == 1:
                out[d.name] = gwfl.FieldInfo(d.name, "nodal", 1, slot=d.slot)
            else:
                raise L.UnsupportedExpression(
                    L.E_UNSUPPORTED, f"{d.name}: only P0 data or data on the variable's FEM")
        return out

    def add_expression(self, expr: str, mim: MeshIm, region: int = -1,
                       add_derivative_order: int = 2) -> int:
        if region != -1:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "regions other than all convexes")
        vars_ = [d for d in self.data.values() if d.kind == "variable"]
        if len(vars_) != 1:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "exactly one fem variable is needed")
        var = vars_[0]
        if var.mf.mesh is not mim.mesh:
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, "mim and variable on different meshes")
        info = gwfl.FieldInfo(var.name, "variable", var.mf.qdim, slot=L.SLOT_U)
        low = gwfl.lower(expr, info, mim.mesh.dim, self._field_infos(var), add_derivative_order)
        g = next((g for g in self.groups if g.var is var and g.mim is mim), None)
        if g is None:
            g = _Group(var, mim)
            self.groups.append(g)
        if low.internal is not None:
            if self.data[low.internal["name"]].imd.mim is not mim:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                              "internal variable on another integration method")
            if g.internal and g.internal["name"] != low.internal["name"]:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED, "one internal variable per group")
            for k, v in low.internal.items():
                if k in g.internal and k != "name":
                    raise L.UnsupportedExpression(
                        L.E_UNSUPPORTED, f"the {'displacement' if k == 'sp' else 'internal'} "
                        "equation of the internal variable is given twice")
                g.internal[k] = v
        g.order2 += low.order2
        g.order1 += low.order1
        g.order0 += low.order0
        return low.max_order

    def tune(self, reps: int = 3):
        """Autotunes the launch configuration (threads per element of the
        element pass, warps per block of the row gather) of the K + R plan
        of every group (gfgpu_tune) and returns {group index: (ep_threads,
        gather_warps)}; later plans of the same element family on this GPU
        model start with it.  Results are the same bits for every
        configuration."""
        lib = L.lib()
        out = {}
        for i, g in enumerate(self.groups):
            if not g.order1:
                continue
            h = self._plan(g, g.order1)
            self._upload(h, g.order1, need_u=True)
            best = L.Launch()
            L.check(lib.gfgpu_tune(h, int(reps), C.byref(best)))
            out[i] = (best.ep_threads, best.gather_warps)
        return out

    def clear_expressions(self):
        self._destroy()
        self.groups = []

    # ------------------------------------------------------------ assembly
    def set_assembled_matrix(self, K):
        self._ext_K = K

    def set_assembled_vector(self, V):
        self._ext_V = V

    def set_internal_coupling_matrix(self, KQJ):
        self._ext_KQJ = KQJ

    def _plan(self, g: _Group, terms):
        key = _terms_key(terms)
        if key in g.plans:
            return g.plans[key]
        mf, mim = g.var.mf, g.mim
        m = mf.mesh
        sp = L.Space()
        sp.dim, sp.kind, sp.degree, sp.qdim = m.dim, m.kind, mf.degree, mf.qdim
        sp.im = mim.im.encode()
        sp.n_points, sp.n_elements, sp.n_dof = m.nb_points(), m.nb_convex(), mf.nb_dof()
        sp.points = m.points.ctypes.data_as(C.POINTER(C.c_double))
        sp.cvpts = m.cvpts.ctypes.data_as(C.POINTER(C.c_int64))
        sp.dofs = mf.dofs.ctypes.data_as(C.POINTER(C.c_int64))
        form = gwfl.to_form(terms)
        h = C.c_void_p()
        stream = None if self._stream is None else C.c_void_p(self._stream)
        L.check(L.lib().gfgpu_plan_create(C.byref(sp), C.byref(form), stream, C.byref(h)))
        g.plans[key] = h
        self._plans.append(h)
        return h

    def _upload(self, h, terms, need_u: bool):
        lib = L.lib()
        used = set()
        for t in terms:
            for c in t["c"]:
                if c is not None and c["kind"] in (L.COEF_ELEMENT, L.COEF_NODAL):
                    used.add(c["slot"])
            if t["kind"] in (L.TERM_SOURCE, L.TERM_INTERNAL_P):
                used.add(t["field_slot"])
        if need_u or any(t["kind"] == L.TERM_NEOHOOKEAN for t in terms):
            used.add(L.SLOT_U)
        for d in self.data.values():
            if d.slot in used:
                self._set_slot(h, d.slot, d.values)

    @staticmethod
    def _set_slot(h, slot, values):
        lib = L.lib()
        if _is_torch_cuda(values):
            v = values.contiguous()
            L.check(lib.gfgpu_set_data(h, slot, C.c_void_p(v.data_ptr()), v.numel(), 1))
        else:
            v = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
            L.check(lib.gfgpu_set_data(h, slot, v.ctypes.data_as(C.c_void_p), v.size, 0))
            L.check(lib.gfgpu_sync(h))

    def assembly(self, order: int, condensation: bool = False):
        if order not in (0, 1, 2):
            raise ValueError("order must be 0, 1 or 2")
        lib = L.lib()
        n = None
        results = []
        pot = 0.0
        cond = []  # (plan, group) of the condensed groups
        for g in self.groups:
            terms = (g.order0, g.order1, g.order2)[order]
            ip = g.internal_term(self) if order > 0 else None
            if ip is not None and order == 1 and not condensation:
                raise L.GfgpuError(L.E_INVALID, "the residual of an internal variable needs "
                                   "condensation=True (its rows follow the primary ones)")
            if ip is not None and (order == 1 or condensation):
                terms = terms + [ip]
            if not terms:
                continue
            h = self._plan(g, terms)
            self._upload(h, terms, need_u=(order <= 1 or ip is not None))
            if order == 0:
                e = C.c_double()
                L.check(lib.gfgpu_assemble(h, 0, 0, C.byref(e)))
                pot += e.value
                continue
            flags = 0
            if ip is not None and order == 2:
                # the internal rows of the current assembled vector are the
                # residual the condensation reads (workspace.cc:826-833)
                nu = g.var.mf.nb_dof()
                cur = self._ext_V if self._ext_V is not None else self._V
                nint = self.nb_internal_dof()
                if cur is None or len(cur) != nu + nint:
                    raise L.GfgpuError(L.E_STATE, "condensation reads the residual of the "
                                       "internal variable from the assembled vector: assemble "
                                       f"order 1 with condensation first (size {nu + nint})")
                self._set_slot(h, ip["aux_slot"], np.asarray(cur)[nu:])
                flags = L.CONDENSATION
            L.check(lib.gfgpu_assemble(h, order, flags, None))
            L.check(lib.gfgpu_sync(h))
            n = g.var.mf.nb_dof()
            results.append(h)
            if ip is not None:
                cond.append(h)
        if order == 0:
            # accumulated like the reference's assembled_potential
            self._E = pot
        elif order == 2:
            self._K = self._collect_matrix(results, n)
            if self._ext_K is not None and self._K is not None:
                self._ext_K += self._K
            if cond:
                # the vector is overwritten: the condensed primary rows, then
                # the internal solution
                V = np.concatenate([self._collect_vector(cond, n), self._collect_internal(cond)])
                self._V = V
                if self._ext_V is not None:
                    self._ext_V[:] = V
                self._KQJ = self._collect_coupling(cond, n)
                if self._ext_KQJ is not None:
                    self._ext_KQJ += self._KQJ
        else:
            self._V = self._collect_vector(results, n)
            if cond:
                self._V = np.concatenate([self._V, self._collect_internal(cond)])
            if self._ext_V is not None and self._V is not None:
                self._ext_V += self._V

    def _collect_internal(self, plans):
        lib = L.lib()
        out = None
        for h in plans:
            ni, rl = C.c_int64(), C.c_int64()
            L.check(lib.gfgpu_internal_size(h, C.byref(ni), C.byref(rl)))
            v = np.empty(ni.value)
            L.check(lib.gfgpu_copy_result(h, L.RESULT_INTERNAL, v.ctypes.data_as(C.c_void_p)))
            out = v if out is None else out + v
        return out

    def _collect_coupling(self, plans, n):
        """KQJpr as a scipy CSR of (n + n_int) x n, the internal rows last
        (getfem_generic_assembly.h:414-419)."""
        import scipy.sparse as sp
        lib = L.lib()
        M = None
        for h in plans:
            ni, rl = C.c_int64(), C.c_int64()
            L.check(lib.gfgpu_internal_size(h, C.byref(ni), C.byref(rl)))
            vals = np.empty(ni.value * rl.value)
            cols = np.empty(ni.value * rl.value, dtype=np.int32)
            L.check(lib.gfgpu_copy_result(h, L.RESULT_COUPLING, vals.ctypes.data_as(C.c_void_p)))
            L.check(lib.gfgpu_copy_result(h, L.RESULT_COUPLING_COLIDX,
                                          cols.ctypes.data_as(C.c_void_p)))
            rowptr = np.concatenate([np.zeros(n, dtype=np.int64),
                                     np.arange(ni.value + 1, dtype=np.int64) * rl.value])
            A = sp.csr_matrix((vals, cols, rowptr), shape=(n + ni.value, n))
            A.sum_duplicates()
            A.sort_indices()
            M = A if M is None else M + A
        return M

    def internal_coupling_matrix(self):
        return self._KQJ

    def _collect_matrix(self, plans, n):
        import scipy.sparse as sp
        lib = L.lib()
        K = None
        for h in plans:
            nr, nnz = C.c_int64(), C.c_int64()
            L.check(lib.gfgpu_pattern_size(h, C.byref(nr), C.byref(nnz)))
            rowptr = np.empty(nr.value + 1, dtype=np.int64)
            colidx = np.empty(nnz.value, dtype=np.int32)
            vals = np.empty(nnz.value)
            for which, arr in ((0, rowptr), (1, colidx), (2, vals)):
                L.check(lib.gfgpu_copy_result(h, which, arr.ctypes.data_as(C.c_void_p)))
            M = sp.csr_matrix((vals, colidx, rowptr), shape=(nr.value, nr.value))
            K = M if K is None else K + M
        return K

    def _collect_vector(self, plans, n):
        lib = L.lib()
        V = None
        for h in plans:
            v = np.empty(n)
            L.check(lib.gfgpu_copy_result(h, 3, v.ctypes.data_as(C.c_void_p)))
            V = v if V is None else V + v
        return V

    def assembled_matrix(self):
        return self._K

    def assembled_vector(self):
        return self._V

    def assembled_potential(self):
        return self._E

    def plans(self):
        """Raw plan handles (for device-side access through the C ABI)."""
        return list(self._plans)

    def _destroy(self):
        if L._lib is not None:
            for h in self._plans:
                L.lib().gfgpu_plan_destroy(h)
        self._plans = []

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass
