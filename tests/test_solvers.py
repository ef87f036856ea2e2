"""Boundary DOFs (host) and the device linear solve of the 2-D Poisson
problem: Dirichlet elimination + CG against the reference's own gmm::cg
solution on the same eliminated system (tests/golden/p1tri_poisson_cg.npz)."""
import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import solvers

from common import build_case, load


def test_boundary_dofs_match_reference():
    rec = load("p1tri_poisson_cg")
    mesh, mf, mim, ws = build_case(rec)
    assert np.array_equal(solvers.boundary_dofs(mf), np.sort(rec["dirichlet"]))


@pytest.mark.parametrize("kind,qdim,deg", [("simplex", 3, 2), ("hex", 1, 2), ("hex", 3, 1)])
def test_boundary_dofs_are_the_boundary_nodes(kind, qdim, deg):
    mesh = g.Mesh.regular_unit(3, 3, kind)
    mf = g.MeshFem(mesh, qdim, degree=deg)
    xyz = mf.basic_dof_nodes()
    on = np.any((np.abs(xyz) < 1e-12) | (np.abs(xyz - 1) < 1e-12), axis=1)
    expect = np.sort((np.nonzero(on)[0][:, None] * qdim + np.arange(qdim)).ravel())
    assert np.array_equal(solvers.boundary_dofs(mf), expect)


@pytest.mark.gpu
@pytest.mark.parametrize("precond", ["identity", "diagonal"])
def test_poisson_cg_matches_reference(precond):
    torch = pytest.importorskip("torch")
    rec = load("p1tri_poisson_cg")
    mesh, mf, mim, ws = build_case(rec)
    dofs = solvers.boundary_dofs(mf)
    u, info = solvers.solve_linear(ws, dofs, resmax=1e-12, precond=precond)
    x = u.cpu().numpy()
    xr = rec["x"]
    assert np.abs(x - xr).max() <= 1e-9 * np.abs(xr).max()
    assert info["residual"] <= 1e-12
    if precond == "identity":
        # the same recurrence as gmm::cg: the iteration count agrees up to
        # the rounding of the dot products
        assert abs(info["iterations"] - int(rec["cg_iterations"][0])) <= 3
        u2, info2 = solvers.solve_linear(ws, dofs, resmax=1e-12, precond=precond)
        assert torch.equal(u, u2) and info2["iterations"] == info["iterations"]


@pytest.mark.gpu
def test_cg_runs_past_one_launch_segment():
    """A small system's CG runs in one block, at most 2000 iterations per
    launch, the host relaunching from the saved recurrence state.  With
    resmax = 0 the solve only stops when the residual is exactly zero (here
    after more than one launch); the solution is that of the converged solve,
    and the run is reproducible bit for bit."""
    torch = pytest.importorskip("torch")
    rec = load("p1tri_poisson_cg")
    mesh, mf, mim, ws = build_case(rec)
    dofs = solvers.boundary_dofs(mf)
    u1, info1 = solvers.solve_linear(ws, dofs, resmax=1e-12)
    u2, info2 = solvers.solve_linear(ws, dofs, resmax=0.0, maxiter=45000)
    u3, info3 = solvers.solve_linear(ws, dofs, resmax=0.0, maxiter=45000)
    assert info2["iterations"] > 2000 and info3["iterations"] == info2["iterations"]
    assert torch.equal(u2, u3)
    x1, x2 = u1.cpu().numpy(), u2.cpu().numpy()
    assert np.abs(x2 - x1).max() <= 1e-9 * np.abs(x1).max()
