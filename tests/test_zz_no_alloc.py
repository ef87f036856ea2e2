"""The allocation-free vector assembly (gfgpu_assemble_vector_noalloc), for
callers that must not allocate device memory themselves (their device memory
belongs to another allocator or to a fixed arena), against the plan entry
point and the oracle: same vector within the suite's tolerance, on two calls
in a row.  The argument checks run on the CPU: a caller's mistake must come
back as GFGPU_E_INVALID before anything is launched.

Collected last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import getfem_gb300 as g
from getfem_gb300 import _lib as L
from getfem_gb300 import gwfl

from common import RTOL, oracle_problem, slots_of, vec_errors


def _problem(nx=5, seed=21):
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
    mf = g.MeshFem(mesh, 3, fem="FEM_PK(3,2)")
    mf0 = g.MeshFem(mesh, 1, fem="FEM_PK(3,0)")
    mim = g.MeshIm(mesh, "IM_TETRAHEDRON(5)")
    E = mesh.nb_convex()
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=rng.standard_normal(mf.nb_dof()) * 0.01)
    ws.add_fem_constant("lambda", mf0, np.exp(rng.normal(0, 0.2, E)))
    ws.add_fem_constant("mu", mf0, np.exp(rng.normal(0, 0.2, E)))
    ws.add_fem_constant("f", mf, rng.standard_normal(mf.nb_dof()))
    ws.add_expression("(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u", mim)
    return mesh, mf, mim, ws


def _adjacency(enode, n_nodes):
    """node -> element*nb + local node, ascending element order (counting sort)."""
    E, nb = enode.shape
    flat = enode.ravel()
    order = np.argsort(flat, kind="stable")  # stable: element order kept per node
    ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.add.at(ptr, flat + 1, 1)
    return np.cumsum(ptr).astype(np.int32), order.astype(np.int32)


@pytest.mark.gpu
def test_noalloc_vector_matches_plan_vector_twice():
    torch = pytest.importorskip("torch")
    mesh, mf, mim, ws = _problem()
    ws.assembly(1)
    R_plan = ws.assembled_vector()

    dev = torch.device("cuda", 0)
    qd = mf.qdim
    enode = (mf.dofs // qd).astype(np.int32)
    n_nodes = mf.nb_dof() // qd
    adj_ptr, adj = _adjacency(enode, n_nodes)
    keep = []

    def dptr(a, dtype):
        t = torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).to(dev)
        keep.append(t)
        return t.data_ptr()

    args = L.NoallocArgs()
    args.dim, args.degree, args.qdim = 3, 2, qd
    args.im = mim.im.encode()
    args.n_elements, args.n_nodes = mesh.nb_convex(), n_nodes
    args.points = dptr(mesh.points, np.float64)
    args.cvpts = dptr(mesh.cvpts, np.int32)
    args.enode = dptr(enode, np.int32)
    args.adj_ptr = dptr(adj_ptr, np.int32)
    args.adj = dptr(adj, np.int32)
    for d in ws.data.values():
        if d.slot >= 0:
            args.slots[d.slot] = dptr(np.asarray(d.values, dtype=np.float64), np.float64)
    out = torch.full((mf.nb_dof(),), float("nan"), dtype=torch.float64, device=dev)
    args.vec = out.data_ptr()
    form = gwfl.to_form(ws.groups[0].order1)
    lib = L.lib()
    results = []
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        L.check(lib.gfgpu_assemble_vector_noalloc(C.byref(args), C.byref(form), None))
        results.append(out.cpu().numpy().copy())
    R_oracle = oracle_problem(mesh, mf, mim, ws.groups[0].order1, slots_of(ws)).vector(nthreads=1)
    for R in results:
        assert vec_errors(R, R_plan).max() <= RTOL
        assert vec_errors(R, R_oracle).max() <= RTOL
    assert np.array_equal(results[0], results[1])


def _valid_args(n_elements=10, n_nodes=10):
    """Arguments that pass every host check; the pointers are dummies that no
    test lets reach a launch."""
    args = L.NoallocArgs()
    args.dim, args.degree, args.qdim = 3, 2, 3
    args.im = b"IM_TETRAHEDRON(5)"
    args.n_elements, args.n_nodes = n_elements, n_nodes
    args.points = args.cvpts = args.enode = args.adj_ptr = args.adj = args.vec = 1
    args.slots[0] = 1
    return args


def _elasticity_form(coef_slot=1, source_slot=3):
    form = L.Form()
    form.n_terms = 2
    t = form.terms[0]
    t.kind, t.scale = 1, 1.0  # GRADGRAD
    t.c[0].kind, t.c[0].slot, t.c[0].value = 2, coef_slot, 1.0  # ELEMENT
    t.c[1].kind, t.c[1].value = 1, 1.0  # CONST
    t.c[2].kind, t.c[2].value = 1, 1.0
    s = form.terms[1]
    s.kind, s.scale, s.field_slot = 3, -1.0, source_slot  # SOURCE
    return form


def _status(args, form):
    return L.lib().gfgpu_assemble_vector_noalloc(C.byref(args), C.byref(form), None)


def test_noalloc_rejects_meshes_beyond_its_scratch():
    args = _valid_args()
    args.n_elements = L.NOALLOC_SCRATCH_BYTES // (32 * 8) + 1
    args.slots[1] = args.slots[3] = 1
    assert _status(args, _elasticity_form()) == L.E_INVALID
    assert b"GFGPU_NOALLOC_SCRATCH_BYTES" in L.lib().gfgpu_last_error()


def test_noalloc_rejects_a_missing_coefficient_slot():
    args = _valid_args()
    args.slots[3] = 1  # the load is there, the per-element coefficient (slot 1) is not
    assert _status(args, _elasticity_form()) == L.E_INVALID
    assert b"coefficient slot" in L.lib().gfgpu_last_error()


def test_noalloc_rejects_a_coefficient_slot_out_of_range():
    args = _valid_args()
    args.slots[3] = 1
    assert _status(args, _elasticity_form(coef_slot=L.MAX_SLOTS)) == L.E_INVALID


def test_noalloc_rejects_a_missing_source_field():
    args = _valid_args()
    args.slots[1] = 1
    assert _status(args, _elasticity_form()) == L.E_INVALID
    assert b"source field" in L.lib().gfgpu_last_error()


def test_noalloc_rejects_too_many_terms():
    args = _valid_args()
    args.slots[1] = args.slots[3] = 1
    form = _elasticity_form()
    form.n_terms = 9
    assert _status(args, form) == L.E_INVALID
    assert b"terms" in L.lib().gfgpu_last_error()


def test_noalloc_rejects_null_adjacency_without_elements():
    """No elements but nodes to write: the adjacency and the output must
    still be real pointers."""
    args = _valid_args(n_elements=0, n_nodes=4)
    args.adj_ptr = None
    assert _status(args, _elasticity_form()) == L.E_INVALID
    args = _valid_args(n_elements=0, n_nodes=4)
    args.vec = None
    assert _status(args, _elasticity_form()) == L.E_INVALID




def test_noalloc_refuses_an_anisotropic_coupling():
    """The allocation-free pass has no anisotropic-coupling instances: a form
    with a GRADGRAD_TENSOR term is refused, not assembled without it."""
    args = _valid_args()
    args.slots[1] = args.slots[3] = 1
    form = _elasticity_form()
    t = form.terms[2]
    t.kind, t.scale = L.TERM_GRADGRAD_TENSOR, 1.0
    for i in range(9):
        form.tensor[i * 9 + i] = 1.0
    form.n_terms = 3
    assert _status(args, form) == L.E_UNSUPPORTED
    assert b"anisotropic" in L.lib().gfgpu_last_error()
    # an unsymmetric tensor is refused by the form check itself
    form.tensor[1] = 0.5
    assert _status(args, form) == L.E_UNSUPPORTED
    assert b"symmetric" in L.lib().gfgpu_last_error()
