"""Sizes of the reference tables used by the kernels (host side)."""
from __future__ import annotations

from itertools import product


def simplex_term_count(dim: int, degree: int, im: str | None = None):
    """Total number of terms of the sparse barycentric reference tensor of
    FEM_PK(dim, degree), summed over local node pairs (i, j), and the number
    of local nodes: grad phi_i involves the barycentric coordinates with a
    nonzero weight in node i, so pair (i, j) has |supp(i)| |supp(j)| terms."""
    supp = []
    for c in product(range(degree + 1), repeat=dim):
        if sum(c) > degree:
            continue
        w = [degree - sum(c)] + list(c)
        supp.append(sum(1 for x in w if x > 0))
    s = sum(supp)
    return s * s, len(supp)


def simplex_upper_term_count(dim: int, degree: int) -> int:
    """Terms over the node pairs i <= j (the symmetric element pass computes
    each pair block once): ((sum |supp|)^2 + sum |supp|^2) / 2."""
    supp = []
    for c in product(range(degree + 1), repeat=dim):
        if sum(c) > degree:
            continue
        w = [degree - sum(c)] + list(c)
        supp.append(sum(1 for x in w if x > 0))
    return (sum(supp) ** 2 + sum(x * x for x in supp)) // 2
