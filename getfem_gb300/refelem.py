"""Reference-element helpers on the host (node coordinates, geometric
basis) used to place DOF nodes for interpolating data fields."""
from __future__ import annotations

import numpy as np

from . import _lib as L


def lagrange_nodes(dim: int, kind: int, degree: int) -> np.ndarray:
    """Reference nodes of FEM_PK/QK(dim, degree) in GetFEM's order (first
    coordinate fastest; simplex lattice points with sum <= degree)."""
    if degree == 0:
        c = 1.0 / (dim + 1) if kind == L.SIMPLEX else 0.5
        return np.full((1, dim), c)
    K = degree
    out = []
    rng = [range(K + 1)] * dim + [range(1)] * (3 - dim)
    for c2 in rng[2]:
        for c1 in rng[1]:
            for c0 in rng[0]:
                c = [c0, c1, c2][:dim]
                if kind == L.SIMPLEX and sum(c) > K:
                    continue
                out.append([x / K for x in c])
    return np.array(out, dtype=float)


def geo_basis(dim: int, kind: int, x: np.ndarray) -> np.ndarray:
    """Values of the GT_PK(dim,1) / GT_QK(dim,1) basis at points x (n x dim):
    returns n x nbg."""
    x = np.asarray(x, dtype=float)
    if kind == L.SIMPLEX:
        return np.concatenate([1.0 - x.sum(axis=1, keepdims=True), x], axis=1)
    cols = []
    for p in range(2 ** dim):
        v = np.ones(x.shape[0])
        for d in range(dim):
            v = v * (x[:, d] if (p >> d) & 1 else 1.0 - x[:, d])
        cols.append(v)
    return np.stack(cols, axis=1)
