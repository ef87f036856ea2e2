"""gf.asm('generic', ...) on the GPU backend.

Mirrors the interface's high-level generic assembly
(interface/src/gf_asm.cc:421-560): a mesh_im, an order, a GWFL expression,
a region, then for every datum a (name, is_variable, mesh_fem or nothing,
values) group; variables become fem variables and the rest fem or
fixed-size constants of a fresh workspace; the expression is added with
derivative order 2 (0 for order 0) and assembled.  Returns the potential
(order 0), the residual vector (order 1) or the sparse matrix (order 2,
scipy CSR).  The select_output and Secondary_domain options are not
lowered.
"""
from __future__ import annotations

from . import _lib as L
from .mesh import MeshFem
from .workspace import GaWorkspace


def asm_generic(mim, order: int, expr: str, region: int = -1, *args):
    if order not in (0, 1, 2):
        raise ValueError("Invalid order, should be 0, 1 or 2")
    ws = GaWorkspace()
    rest = list(args)
    seen = set()
    while rest:
        name = rest.pop(0)
        if name in ("select_output", "select output", "Secondary_domain", "Secondary_Domain"):
            raise L.UnsupportedExpression(L.E_UNSUPPORTED, f"option {name!r} is not lowered")
        if name in seen:
            raise ValueError(f"The same variable/constant name is repeated twice: {name}")
        seen.add(name)
        is_var = int(rest.pop(0)) != 0
        mf = rest.pop(0) if rest and isinstance(rest[0], MeshFem) else None
        values = rest.pop(0)
        if is_var:
            if mf is None:
                raise L.UnsupportedExpression(L.E_UNSUPPORTED,
                                              "fixed-size and im_data variables are not lowered")
            ws.add_fem_variable(name, mf, U=values)
        elif mf is not None:
            ws.add_fem_constant(name, mf, values)
        else:
            ws.add_fixed_size_constant(name, values)
    ws.add_expression(expr, mim, region, 2 if order else 0)
    ws.assembly(order)
    if order == 0:
        return ws.assembled_potential()
    if order == 1:
        return ws.assembled_vector()
    return ws.assembled_matrix()
