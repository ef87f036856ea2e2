"""Differentiable potentials: the workspace's order-0 assembly as a torch
function of the variable u, of per-element or nodal coefficient data and of
the mesh vertex coordinates.

    pot = Potential(ws)                      # ws holds a potential expression
    E = pot(u, points=X, mu=mu)              # torch scalar (float64, CUDA)
    E.backward()                             # u.grad, X.grad, mu.grad

Forward is gfgpu_assemble(order 0); backward is the order-1 assembly of the
same expression for u (GWFL's derivative of the potential, which the
reference obtains with assembly(1) of the potential,
getfem_generic_assembly_workspace.cc:791), and gfgpu_potential_gradient for
the coefficient data and the coordinates (the shape derivative with the DOF
values held fixed).  All tensors stay on the device.
"""
from __future__ import annotations

import ctypes as C

from . import _lib as L


def _torch():
    import torch
    return torch


class Potential:
    """The potential of one (variable, integration method) group of a
    GaWorkspace, callable on torch CUDA tensors."""

    def __init__(self, ws, group: int = 0):
        self.ws = ws
        self.g = ws.groups[group]
        if not self.g.order0:
            raise ValueError("the workspace holds no potential expression")
        self.h0 = ws._plan(self.g, self.g.order0)
        self.h1 = ws._plan(self.g, self.g.order1) if self.g.order1 else None
        self.mf = self.g.var.mf
        self.mesh = self.mf.mesh

    def __call__(self, u, points=None, **fields):
        names = sorted(fields)
        return _PotentialFn.apply(self, names, u, points, *[fields[n] for n in names])

    # -- plumbing
    def _bind(self, h, u, points, names, vals):
        lib = L.lib()
        self.ws._set_slot(h, L.SLOT_U, u)
        for nm, v in zip(names, vals):
            d = self.ws.data[nm]
            self.ws._set_slot(h, d.slot, v)
        # data of the workspace that the caller did not pass
        for d in self.ws.data.values():
            if d.slot > 0 and d.name not in names and d.kind != "variable":
                self.ws._set_slot(h, d.slot, d.values)
        if points is not None:
            p = points.contiguous()
            L.check(lib.gfgpu_set_points(h, C.c_void_p(p.data_ptr()), p.numel(), 1))


class _PotentialFn:
    """torch.autograd.Function, created lazily so that importing the package
    does not import torch."""
    _cls = None

    @classmethod
    def apply(cls, *args):
        if cls._cls is None:
            cls._cls = _make_function()
        return cls._cls.apply(*args)


def _make_function():
    torch = _torch()

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pot, names, u, points, *vals):
            lib = L.lib()
            u = u.contiguous()
            vals = [v.contiguous() for v in vals]
            pot._bind(pot.h0, u, points, names, vals)
            e = C.c_double()
            L.check(lib.gfgpu_assemble(pot.h0, 0, 0, C.byref(e)))
            ctx.pot, ctx.names = pot, names
            ctx.save_for_backward(u, points if points is not None else torch.empty(0), *vals)
            ctx.has_points = points is not None
            return torch.tensor(e.value, dtype=torch.float64, device=u.device)

        @staticmethod
        def backward(ctx, gE):
            lib = L.lib()
            pot, names = ctx.pot, ctx.names
            u, points, *vals = ctx.saved_tensors
            points = points if ctx.has_points else None
            g_u = g_p = None
            g_vals = [None] * len(vals)
            if ctx.needs_input_grad[2]:
                if pot.h1 is None:
                    raise RuntimeError("no order-1 form for the variable")
                pot._bind(pot.h1, u, points, names, vals)
                L.check(lib.gfgpu_assemble(pot.h1, 1, 0, None))
                g_u = torch.empty_like(u)
                L.check(lib.gfgpu_copy_result(pot.h1, L.RESULT_VECTOR,
                                              C.c_void_p(g_u.data_ptr())))
                g_u = g_u * gE
            pot._bind(pot.h0, u, points, names, vals)
            if ctx.has_points and ctx.needs_input_grad[3]:
                g_p = torch.empty_like(points)
                L.check(lib.gfgpu_potential_gradient(pot.h0, L.SLOT_POINTS,
                                                     C.c_void_p(g_p.data_ptr()), g_p.numel(), 1))
                g_p = g_p * gE
            for i, (nm, v) in enumerate(zip(names, vals)):
                if ctx.needs_input_grad[4 + i]:
                    g = torch.empty_like(v)
                    L.check(lib.gfgpu_potential_gradient(pot.h0, pot.ws.data[nm].slot,
                                                         C.c_void_p(g.data_ptr()), g.numel(), 1))
                    g_vals[i] = g * gE
            return (None, None, g_u, g_p, *g_vals)

    return Fn
