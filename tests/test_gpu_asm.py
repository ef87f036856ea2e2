"""asm_generic (the gf.asm('generic', ...) call) against the reference
fixtures: the matrix, the residual and the potential of the same data."""
import numpy as np
import pytest

import getfem_gb300 as g

from common import RTOL, assert_same_pattern, golden_csr, load, value_errors, vec_errors

pytestmark = pytest.mark.gpu


def fixture_args(rec):
    m = rec["meta"]
    kind = "simplex" if m["gt"] == "PK" else "hex"
    mesh = g.Mesh.regular_unit(m["dim"], m["nx"], kind, jitter=rec.get("jitter"))
    mf = g.MeshFem(mesh, m["qdim"], degree=m["degree"])
    mim = g.MeshIm(mesh, m["im"])
    args = ["u", 1, mf, rec["in_u"]]
    for cname, ck in m["consts"].items():
        v = rec["in_" + cname]
        if ck == "P0":
            args += [cname, 0, g.MeshFem(mesh, 1, degree=0), v]
        elif ck == "V":
            args += [cname, 0, mf, v]
        elif ck == "S":
            args += [cname, 0, g.MeshFem(mesh, 1, degree=m["degree"]), v]
        else:
            args += [cname, 0, v]
    return mim, m["expr"], args


@pytest.mark.parametrize("name", ["p2tet_elastic", "q2hex_neohookean", "p2tri_energy_potential"])
def test_asm_generic_matches_reference(name):
    rec = load(name)
    mim, expr, args = fixture_args(rec)
    K = g.asm_generic(mim, 2, expr, -1, *args)
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    R = g.asm_generic(mim, 1, expr, -1, *args)
    assert vec_errors(R, rec["R"]).max() <= RTOL
    if "E" in rec:
        E = g.asm_generic(mim, 0, expr, -1, *args)
        assert abs(E - float(rec["E"][0])) <= RTOL * abs(float(rec["E"][0]))


def test_asm_generic_rejects_unlowered_options():
    rec = load("p1tri_poisson")
    mim, expr, args = fixture_args(rec)
    with pytest.raises(g.UnsupportedExpression):
        g.asm_generic(mim, 2, expr, -1, *args, "select_output", "u", "u")
