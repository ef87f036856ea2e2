"""Pins the oracle (oracle/gfref.cc, a CPU restatement of the reference's
exec loop) against the reference's own assembly of the same expressions:
sparsity pattern bit-exact, K and R within 1e-12 relative, potentials
(order 0) within 1e-12 relative."""
import numpy as np
import pytest

from common import (RTOL, assert_same_pattern, build_case, golden_csr, golden_names, load,
                    oracle_problem, slots_of, value_errors, vec_errors)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_case(rec)
    grp = ws.groups[0]
    slots = slots_of(ws)
    K = oracle_problem(mesh, mf, mim, grp.order2, slots).matrix(nthreads=1)
    Kref = golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    R = oracle_problem(mesh, mf, mim, grp.order1, slots).vector(nthreads=1)
    assert vec_errors(R, rec["R"]).max() <= RTOL
    if "E" in rec:
        E = oracle_problem(mesh, mf, mim, grp.order0, slots).potential(nthreads=1)
        assert abs(E - float(rec["E"][0])) <= RTOL * abs(float(rec["E"][0]))


def test_oracle_threads_agree():
    rec = load("p2tet_elastic")
    mesh, mf, mim, ws = build_case(rec)
    grp = ws.groups[0]
    P = oracle_problem(mesh, mf, mim, grp.order2, slots_of(ws))
    K1 = P.matrix(nthreads=1)
    K4 = P.matrix(nthreads=4)
    assert_same_pattern(K1, K4)
    assert value_errors(K4, K1).max() <= RTOL
