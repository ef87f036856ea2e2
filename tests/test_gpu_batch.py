"""Batched multi-mesh assembly: one persistent launch over a mix of P1/P2
triangle Poisson and P1/P2 tetrahedron elasticity meshes gives, mesh by
mesh, bit for bit the K and R of the single-mesh path; a CUDA graph of the
batched assembly replayed with coefficients perturbed in place matches the
single-mesh assembly with the same coefficients."""
import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300.batch import Batch

pytestmark = pytest.mark.gpu

TYPES = [("tri", 1), ("tri", 2), ("tet", 1), ("tet", 2)]


def make_ws(kind, degree, nx, seed, torch):
    rng = np.random.default_rng(seed)
    dim = 2 if kind == "tri" else 3
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** dim, dim))
    mesh = g.Mesh.regular_unit(dim, nx, "simplex", jitter=jit)
    qdim = 1 if kind == "tri" else 3
    mf = g.MeshFem(mesh, qdim, degree=degree)
    mf0 = g.MeshFem(mesh, 1, degree=0)
    E = mesh.nb_convex()
    dev = "cuda"
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=torch.tensor(rng.standard_normal(mf.nb_dof()) * 0.1, device=dev))
    coefs = {}
    if kind == "tri":
        coefs["kappa"] = torch.tensor(np.exp(rng.normal(0, 0.2, E)), device=dev)
        ws.add_fem_constant("kappa", mf0, coefs["kappa"])
        ws.add_fem_constant("f", mf, torch.tensor(rng.uniform(-1, 1, mf.nb_dof()), device=dev))
        mim = g.MeshIm(mesh, "IM_TRIANGLE(2)" if degree == 1 else "IM_TRIANGLE(4)")
        ws.add_expression("kappa*Grad_u.Grad_Test_u - f*Test_u", mim)
    else:
        for nm in ("lambda", "mu"):
            coefs[nm] = torch.tensor(np.exp(rng.normal(0, 0.2, E)), device=dev)
            ws.add_fem_constant(nm, mf0, coefs[nm])
        ws.add_fem_constant("f", mf, torch.tensor(rng.standard_normal(mf.nb_dof()), device=dev))
        mim = g.MeshIm(mesh, "IM_TETRAHEDRON(2)" if degree == 1 else "IM_TETRAHEDRON(5)")
        ws.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u", mim)
    return ws, coefs


def single(ws):
    ws.assembly(2)
    K = ws.assembled_matrix().copy()
    ws.assembly(1)
    return K, ws.assembled_vector().copy()


def test_batch_matches_single_mesh_path_bitwise():
    torch = pytest.importorskip("torch")
    wss = []
    for i in range(12):
        kind, deg = TYPES[i % 4]
        nx = [3, 5, 8][i % 3] if kind == "tri" else [2, 3][i % 2]
        wss.append(make_ws(kind, deg, nx, 100 + i, torch)[0])
    ref = [single(ws) for ws in wss]
    b = Batch(wss)
    b.tune()
    b.assemble()
    b.sync()
    for i, (K, R) in enumerate(ref):
        Kb, Rb = b.matrix(i), b.vector(i)
        assert np.array_equal(Kb.indptr, K.indptr) and np.array_equal(Kb.indices, K.indices)
        assert np.array_equal(Kb.data, K.data), i
        # the single-mesh order-1 vector comes from the element pass of the
        # order-1 form: bit-identical to the fused K + R pass is not required
        assert np.allclose(Rb, R, rtol=1e-12, atol=1e-12 * np.abs(R).max())


def test_batch_graph_replay_with_perturbed_coefficients():
    torch = pytest.importorskip("torch")
    pairs = [make_ws(*TYPES[i % 4], 3 if i % 4 < 2 else 2, 200 + i, torch) for i in range(8)]
    wss = [p[0] for p in pairs]
    coefs = [c for p in pairs for c in p[1].values()]
    base = [c.clone() for c in coefs]
    factor = torch.ones(1, dtype=torch.float64, device="cuda")

    def perturb():
        for c, b0 in zip(coefs, base):
            torch.mul(b0, factor, out=c)

    b = Batch(wss)
    graph = b.graph(pre=perturb)
    for rep in range(3):
        factor.fill_(1.0 + 0.05 * (rep + 1))
        graph.replay()
        torch.cuda.synchronize()
        b.sync()
        for i, ws in enumerate(wss):
            K, R = single(ws)  # the workspace reads the same (perturbed) tensors
            assert np.array_equal(b.matrix(i).data, K.data)
