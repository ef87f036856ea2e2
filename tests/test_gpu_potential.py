"""GPU potentials (order-0 assembly) and their adjoints.

Parity: the energy of each potential fixture within 1e-12 of the reference's
assembled_potential, and the reference's own derivatives of the potential
(GWFL Diff: assembly(1) and assembly(2) of the same expression) matched by the
GPU order-1 / order-2 assembly (pattern bit-exact, values within 1e-12).

Adjoint: gradients with respect to u, per-element and nodal coefficients and
the vertex coordinates, through getfem_gb300.Potential (torch autograd),
checked against central finite differences of the GPU potential and of the
oracle's potential, and exactly (1e-12) where the energy is linear in the
datum (E = sum_e theta_e dE/dtheta_e)."""
import numpy as np
import pytest

import getfem_gb300 as g

from common import (RTOL, assert_same_pattern, build_case, golden_csr, load, oracle_problem,
                    slots_of, value_errors, vec_errors)

pytestmark = pytest.mark.gpu

POT_CASES = ["q2hex_nh_potential", "p2tet_nh_potential", "q2hex_kappa_potential",
             "p2tri_energy_potential"]
NH_POT = "Compressible_Neo_Hookean_potential(Grad_u,[0.5*mu;D1])"


@pytest.mark.parametrize("name", POT_CASES)
def test_potential_and_its_derivatives_match_reference(name):
    rec = load(name)
    mesh, mf, mim, ws = build_case(rec)
    ws.assembly(0)
    E, Eref = ws.assembled_potential(), float(rec["E"][0])
    assert abs(E - Eref) <= RTOL * abs(Eref), (E, Eref)
    ws.assembly(2)
    K, Kref = ws.assembled_matrix(), golden_csr(rec)
    assert_same_pattern(K, Kref)
    assert value_errors(K, Kref).max() <= RTOL
    ws.assembly(1)
    assert vec_errors(ws.assembled_vector(), rec["R"]).max() <= RTOL


def _torch():
    return pytest.importorskip("torch")


def nh_problem(kind="hex", nx=2, seed=3):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, kind, jitter=jit)
    mf = g.MeshFem(mesh, 3, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)" if kind == "hex" else "IM_TETRAHEDRON(5)")
    xyz = mf.basic_dof_nodes()
    u = 0.05 * np.sin(xyz @ rng.uniform(-3, 3, (3, 3)) + rng.uniform(0, 6, 3)).ravel()
    mu = np.exp(rng.normal(0, 0.3, mesh.nb_convex()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u)
    ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0), mu)
    ws.add_fixed_size_constant("D1", np.array([1.5]))
    ws.add_expression(NH_POT, mim)
    return rng, mesh, mf, mim, ws, u, mu


@pytest.mark.parametrize("kind", ["hex", "simplex"])
def test_nh_adjoint_against_finite_differences(kind):
    torch = _torch()
    rng, mesh, mf, mim, ws, u0, mu0 = nh_problem(kind)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(u0, device=dev, requires_grad=True)
    X = torch.tensor(mesh.points.ravel(), device=dev, requires_grad=True)
    mu = torch.tensor(mu0, device=dev, requires_grad=True)
    E = pot(u, points=X, mu=mu)
    E.backward()
    gu, gX, gmu = u.grad.clone(), X.grad.clone(), mu.grad.clone()
    E = E.detach()

    def energy(uu, XX, mm):
        with torch.no_grad():
            return float(pot(uu, points=XX, mu=mm))

    # mu enters linearly (C1 = mu / 2): E(mu) - E(0) = sum_e mu_e dE/dmu_e
    E0 = energy(u, X, torch.zeros_like(mu))
    assert abs((float(E) - E0) - float(gmu @ mu)) <= 1e-12 * abs(float(E))
    # directional finite differences in u and in the coordinates
    for grad, name in ((gu, "u"), (gX, "X")):
        d = torch.tensor(rng.standard_normal(grad.numel()), device=dev)
        eps = 1e-6 if name == "u" else 1e-7
        if name == "u":
            fd = (energy(u + eps * d, X, mu) - energy(u - eps * d, X, mu)) / (2 * eps)
        else:
            fd = (energy(u, X + eps * d, mu) - energy(u, X - eps * d, mu)) / (2 * eps)
        an = float(grad @ d)
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3), (name, fd, an)
    # the coordinates gradient against the oracle's potential
    from oracle import gfref
    grp = ws.groups[0]
    slots = slots_of(ws)
    d = rng.standard_normal(mesh.points.size)
    eps = 1e-7

    def e_oracle(pts):
        return gfref.Problem(3, mesh.kind, 2, 3, mim.im, pts.reshape(mesh.points.shape),
                             mesh.cvpts, mf.dofs, mf.nb_dof(), grp.order0, slots).potential(4)
    fd = (e_oracle(mesh.points.ravel() + eps * d) - e_oracle(mesh.points.ravel() - eps * d)) / (2 * eps)
    an = float(gX.cpu().numpy() @ d)
    assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3), (fd, an)


def test_quadratic_potential_adjoint_is_exact():
    """kappa*Grad_u.Grad_u on Q2 hexahedra: dE/du = 2 K u and
    E = sum_e kappa_e dE/dkappa_e, both to 1e-12."""
    torch = _torch()
    rng = np.random.default_rng(8)
    nx = 3
    jit = rng.uniform(-0.1 / nx, 0.1 / nx, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, "hex", jitter=jit)
    mf = g.MeshFem(mesh, 1, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
    u0 = rng.standard_normal(mf.nb_dof())
    k0 = np.exp(rng.normal(0, 0.5, mesh.nb_convex()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u0)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), k0)
    ws.add_expression("kappa*Grad_u.Grad_u", mim)
    ws.assembly(2)
    K = ws.assembled_matrix()
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(u0, device=dev, requires_grad=True)
    kappa = torch.tensor(k0, device=dev, requires_grad=True)
    E = pot(u, kappa=kappa)
    E.backward()
    E = E.detach()
    Ku2 = K @ u0  # K is the second derivative, 2 * (kappa grad grad)
    assert vec_errors(u.grad.cpu().numpy(), Ku2).max() <= RTOL
    assert abs(float(E) - 0.5 * u0 @ Ku2) <= RTOL * abs(float(E))
    assert abs(float(E) - float(kappa.grad @ kappa)) <= RTOL * abs(float(E))


def test_nodal_coefficient_gradient_is_exact():
    torch = _torch()
    rng = np.random.default_rng(12)
    mesh = g.Mesh.regular_unit(2, 6, "simplex",
                               jitter=rng.uniform(-0.015, 0.015, (49, 2)))
    mf = g.MeshFem(mesh, 1, degree=2)
    mim = g.MeshIm(mesh, "IM_TRIANGLE(4)")
    u0 = rng.standard_normal(mf.nb_dof())
    r0 = np.exp(rng.normal(0, 0.3, mf.nb_dof()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u0)
    ws.add_fem_constant("rho", g.MeshFem(mesh, 1, degree=2), r0)
    ws.add_expression("rho*Grad_u.Grad_u + rho*u*u", mim)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    rho = torch.tensor(r0, device=dev, requires_grad=True)
    u = torch.tensor(u0, device=dev)
    E = pot(u, rho=rho)
    E.backward()
    E = E.detach()
    assert abs(float(E) - float(rho.grad @ rho)) <= RTOL * abs(float(E))
    # and against the oracle's potential
    grp = ws.groups[0]
    Eo = oracle_problem(mesh, mf, mim, grp.order0, slots_of(ws)).potential(2)
    assert abs(float(E) - Eo) <= RTOL * abs(Eo)


def test_points_moved_off_parallelepipeds():
    """kappa*Grad_u.Grad_u on Q2 hexahedra of a parallelepiped mesh: the
    order-1/2 plan takes the parallelepiped kernel and the potential forms the
    Jacobian once per element.  Moving an interior vertex (gfgpu_set_points)
    keeps the potential exact (the Jacobian is formed per Gauss point again)
    and makes orders 1 and 2 fail loudly; the original points restore them."""
    import ctypes as C

    from getfem_gb300 import _lib as L
    from oracle import gfref
    torch = _torch()
    rng = np.random.default_rng(12)
    mesh = g.Mesh.regular_unit(3, 2, "hex")
    mf = g.MeshFem(mesh, 1, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
    u0 = rng.standard_normal(mf.nb_dof())
    k0 = np.exp(rng.normal(0, 0.5, mesh.nb_convex()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u0)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), k0)
    ws.add_expression("kappa*Grad_u.Grad_u", mim)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(u0, device=dev)
    kappa = torch.tensor(k0, device=dev)
    X0 = torch.tensor(mesh.points.ravel(), device=dev)
    grp = ws.groups[0]

    def e_oracle(pts):
        return gfref.Problem(3, mesh.kind, 2, 1, mim.im, pts.reshape(mesh.points.shape),
                             mesh.cvpts, mf.dofs, mf.nb_dof(), grp.order0,
                             slots_of(ws)).potential(4)
    E0 = float(pot(u, points=X0, kappa=kappa))
    e0 = e_oracle(mesh.points.ravel())
    assert abs(E0 - e0) <= RTOL * abs(e0), (E0, e0)
    X1 = X0.clone()
    centre = int(np.argmin(np.abs(mesh.points - 0.5).sum(axis=1)))
    X1[3 * centre] += 0.05
    E1 = float(pot(u, points=X1, kappa=kappa))
    e1 = e_oracle(X1.cpu().numpy())
    assert abs(E1 - e1) <= RTOL * abs(e1), (E1, e1)
    assert abs(e1 - e0) > 1e-6 * abs(e0)
    lib = L.lib()
    h1 = pot.h1
    L.check(lib.gfgpu_set_points(h1, C.c_void_p(X1.data_ptr()), X1.numel(), 1))
    assert lib.gfgpu_assemble(h1, 1, 0, None) == L.E_UNSUPPORTED
    assert b"parallelepipeds" in lib.gfgpu_last_error()
    pot._bind(h1, u, X0, ["kappa"], [kappa])
    L.check(lib.gfgpu_assemble(h1, 1, 0, None))
    L.check(lib.gfgpu_sync(h1))


@pytest.mark.parametrize("shear,degree", [(False, 1), (True, 1), (False, 2), (True, 2),
                                          (False, 4), (True, 4)])
def test_parallelepiped_scalar_potential_and_coefficient_gradient(shear, degree):
    """kappa*Grad_u.Grad_u on parallelepiped hexahedra, where the potential
    and dE/dkappa go through the plan's reference tensors: the 3 diagonal
    metric tables on an axis-aligned mesh, all 6 on a sheared one.  E within
    1e-12 of the oracle's potential, and E = sum_e kappa_e dE/dkappa_e."""
    torch = _torch()
    rng = np.random.default_rng(21 + degree + int(shear))
    nx = 3
    mesh = g.Mesh.regular_unit(3, nx, "hex")
    if shear:
        A = np.array([[1.0, 0.3, -0.2], [0.1, 0.9, 0.25], [-0.15, 0.05, 1.1]])
        mesh = g.Mesh(3, mesh.kind, np.ascontiguousarray(mesh.points @ A.T), mesh.cvpts)
    mf = g.MeshFem(mesh, 1, degree=degree)
    im = "IM_GAUSS_PARALLELEPIPED(3,%d)" % {1: 3, 2: 5, 4: 9}[degree]
    mim = g.MeshIm(mesh, im)
    u0 = rng.standard_normal(mf.nb_dof())
    k0 = np.exp(rng.normal(0, 0.5, mesh.nb_convex()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u0)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), k0)
    ws.add_expression("kappa*Grad_u.Grad_u", mim)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(u0, device=dev)
    kappa = torch.tensor(k0, device=dev, requires_grad=True)
    E = pot(u, kappa=kappa)
    E.backward()
    E = E.detach()
    grp = ws.groups[0]
    Eo = oracle_problem(mesh, mf, mim, grp.order0, slots_of(ws)).potential(2)
    assert abs(float(E) - Eo) <= RTOL * abs(Eo), (float(E), Eo)
    assert abs(float(E) - float(kappa.grad @ kappa)) <= RTOL * abs(float(E))


def test_points_moved_onto_parallelepipeds():
    """A potential plan made on a jittered (non-parallelepiped) Q2 mesh whose
    vertices are then moved onto the regular lattice (gfgpu_set_points): the
    plan has no reference tensors, and the energy and dE/dkappa go through the
    Gauss-point sums with several elements per warp.  Both match the oracle
    at the moved points, and E = sum_e kappa_e dE/dkappa_e."""
    from oracle import gfref
    torch = _torch()
    rng = np.random.default_rng(31)
    nx = 3
    jit = rng.uniform(-0.1 / nx, 0.1 / nx, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, "hex", jitter=jit)
    regular = g.Mesh.regular_unit(3, nx, "hex")
    mf = g.MeshFem(mesh, 1, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
    u0 = rng.standard_normal(mf.nb_dof())
    k0 = np.exp(rng.normal(0, 0.5, mesh.nb_convex()))
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u0)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), k0)
    ws.add_expression("kappa*Grad_u.Grad_u", mim)
    pot = g.Potential(ws)
    dev = torch.device("cuda")
    u = torch.tensor(u0, device=dev)
    kappa = torch.tensor(k0, device=dev, requires_grad=True)
    X = torch.tensor(regular.points.ravel(), device=dev)
    E = pot(u, points=X, kappa=kappa)
    E.backward()
    E = E.detach()
    grp = ws.groups[0]
    Eo = gfref.Problem(3, mesh.kind, 2, 1, mim.im, regular.points, mesh.cvpts, mf.dofs,
                       mf.nb_dof(), grp.order0, slots_of(ws)).potential(4)
    assert abs(float(E) - Eo) <= RTOL * abs(Eo), (float(E), Eo)
    assert abs(float(E) - float(kappa.grad @ kappa)) <= RTOL * abs(float(E))
