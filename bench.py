#!/usr/bin/env python3
"""Benchmark of the generic-assembly hot path on GB300.

Workload (one step): value re-assembly of the tangent matrix K and the
residual R of 3-D linear elasticity on a unit cube split into 40^3 x 6
P2 tetrahedra (384 000 elements, 1 594 323 DOFs, IM_TETRAHEDRON(5)), interior
vertices jittered by U[-0.1h, 0.1h], Lame coefficients lambda = mu = 1 each
scaled per element by lognormal(0, 0.2), nodal load N(0, 1):
    (lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u
with the sparsity pattern cached (built once, at warm-up).  Synthetic
seeded data stand in for the reference's configuration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gfgpu|reference]

One JSON line on rank 0.  value = elements/s with inputs resident in HBM;
e2e = the same through the C ABI call with host buffers
(gfgpu_assemble_host: u copied in, K values and R copied out every step).
With N > 1 each rank assembles its own copy of the mesh (replicas: the
path has no exchange step on one node); value sums the ranks' elements over
the slowest rank's time.  --impl reference times the CPU implementation of
the same path (the oracle restatement of the reference's exec loop,
OpenMP over all host cores) on a bounded sub-mesh per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

EXPR = "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u"
METRIC = "elements/s assembled (K + residual), P2 tet elasticity"


# --------------------------------------------------- synthetic inputs
# The inputs are drawn with numpy's Generator (its uniform and normal
# variates are the same bits on every host) and shaped with the two
# functions below instead of np.exp / np.sin, whose last bit differs
# between x86-64 and aarch64 builds of numpy: the fixtures made on one host
# then describe the inputs of the other exactly.  Both use separate IEEE
# multiplies and adds only (numpy ufuncs, never fused), so every host gives
# the same bits; their accuracy is a few units in the last place.

_LN2_HI, _LN2_LO = 0.6931471803691238, 1.9082149292705877e-10  # ln 2 = HI + LO, HI 32 bits
_PIO2 = (1.5707963267341256, 6.077100506303966e-11, 2.0222662487959506e-21)  # pi/2, 3 parts
_INV_FACT = [1.0 / math.factorial(n) for n in range(22)]


def det_exp(x):
    """e^x: x = k ln2 + r, |r| <= ln2/2, e^r by its Taylor series to r^17/17!
    (Horner), scaled by 2^k."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * (1.0 / 0.6931471805599453))
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, _INV_FACT[17])
    for n in range(16, -1, -1):
        p = p * r + _INV_FACT[n]
    return np.ldexp(p, k.astype(np.int64))


def det_sin(t):
    """sin t: t = n pi/2 + r, |r| <= pi/4, then +-sin r or +-cos r by their
    Taylor series (to r^21/21! and r^20/20!)."""
    t = np.asarray(t, dtype=np.float64)
    n = np.rint(t * (2.0 / math.pi))
    r = ((t - n * _PIO2[0]) - n * _PIO2[1]) - n * _PIO2[2]
    r2 = r * r
    s = np.full_like(r, _INV_FACT[21])
    for k in range(19, 0, -2):
        s = s * r2 * (-1.0) + _INV_FACT[k]
    s = s * r
    c = np.full_like(r, _INV_FACT[20])
    for k in range(18, -1, -2):
        c = c * r2 * (-1.0) + _INV_FACT[k]
    q = n.astype(np.int64) % 4
    return np.where(q == 0, s, np.where(q == 1, c, np.where(q == 2, -s, -c)))


def p2tet_inputs(nx: int, seed: int = 2026):
    """Seeded inputs of the P2-tet elasticity workload, made with numpy only
    (the reference arm uses them without the package): interior-vertex
    jitter U[-0.1h, 0.1h] in lattice order (x fastest), u N(0,1)*1e-3, the
    per-element Lame scalings lambda, mu lognormal(0, 0.2) and the nodal load
    f N(0,1).  Sizes of regular_unit_mesh(nx^3) split into 6 tetrahedra
    with FEM_PK(3,2), qdim 3: E = 6 nx^3 elements, 3 (2 nx + 1)^3 DOFs."""
    rng = np.random.default_rng(seed)
    h = 1.0 / nx
    E = 6 * nx ** 3
    ndof = 3 * (2 * nx + 1) ** 3
    jit = rng.uniform(-0.1 * h, 0.1 * h, ((nx + 1) ** 3, 3))
    data = dict(u=rng.standard_normal(ndof) * 1e-3,
                lam=det_exp(rng.normal(0.0, 0.2, E)), mu=det_exp(rng.normal(0.0, 0.2, E)),
                f=rng.standard_normal(ndof))
    return jit, data


def neohookean_inputs(xyz: np.ndarray, E: int, seed: int = 3):
    """Inputs of the Q2 neo-Hookean workload: u = the sum of 8 sinusoid modes
    0.05 sin(k.x + phi) per component (k ~ U[-pi, pi]^3, phi ~ U[0, 2 pi]) at
    the DOF nodes xyz, and the per-element shear modulus lognormal(0, 0.3)."""
    rng = np.random.default_rng(seed)
    u = np.zeros((xyz.shape[0], 3))
    for a in range(3):
        for _ in range(8):
            k = rng.uniform(-np.pi, np.pi, 3)
            t = ((xyz[:, 0] * k[0] + xyz[:, 1] * k[1]) + xyz[:, 2] * k[2]) + rng.uniform(0, 2 * np.pi)
            u[:, a] += 0.05 * det_sin(t)
    mu = det_exp(rng.normal(0, 0.3, E))
    return u.ravel(), mu


def q4_inputs(E: int, ndof: int, seed: int = 5):
    """Inputs of the Q4 Laplacian workload: per-element diffusivity
    lognormal(0, 0.5) and u i.i.d. N(0, 1)."""
    rng = np.random.default_rng(seed)
    kappa = det_exp(rng.normal(0, 0.5, E))
    u = rng.standard_normal(ndof)
    return kappa, u


def poisson_inputs(ndof: int, seed: int = 1):
    """Nodal load of the 2-D Poisson workload, U[-1, 1]."""
    return np.random.default_rng(seed).uniform(-1, 1, ndof)


def make_problem(nx: int, seed: int = 2026):
    import getfem_gb300 as g
    jit, data = p2tet_inputs(nx, seed)
    mesh = g.Mesh.regular_unit(3, nx, "simplex", jitter=jit)
    mf = g.MeshFem(mesh, 3, degree=2)
    mf0 = g.MeshFem(mesh, 1, degree=0)
    mim = g.MeshIm(mesh, "IM_TETRAHEDRON(5)")
    assert mf.nb_dof() == data["u"].size and mesh.nb_convex() == data["lam"].size
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=data["u"])
    ws.add_fem_constant("lambda", mf0, data["lam"])
    ws.add_fem_constant("mu", mf0, data["mu"])
    ws.add_fem_constant("f", mf, data["f"])
    ws.add_expression(EXPR, mim)
    return mesh, mf, mim, ws, data


REF_DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def time_reference_model(nx, threads, warmup, steps, seed=2026):
    """The reference itself (GetFEM built from its sources by
    oracle/refbuild, with OpenMP): model::assembly(BUILD_ALL) of the
    P2-tet elasticity workload (K and the right-hand side; one ga_workspace
    per thread over its partition of the mesh, src/getfem_models.cc:2646-2730)
    on the same seeded inputs, `warmup` untimed then `steps` timed calls with
    steady_clock.  Returns (step seconds list, info dict) or None when the
    reference build is absent."""
    import tempfile
    if not os.access(REF_DRIVER, os.X_OK):
        return None
    jit, data = p2tet_inputs(nx, seed)
    with tempfile.TemporaryDirectory() as td:
        ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        jit.astype(np.float64).tofile(os.path.join(ind, "jitter.bin"))
        for k, name in (("u", "u"), ("lam", "lambda"), ("mu", "mu"), ("f", "f")):
            data[k].astype(np.float64).tofile(os.path.join(ind, name + ".bin"))
        cmd = [REF_DRIVER, "dim=3", f"nx={nx}", "gt=PK", "fem=2", "qdim=3",
               "im=IM_TETRAHEDRON(5)", f"in={ind}", f"out={outd}", f"expr={EXPR}", "jitter=1",
               "consts=lambda:P0,mu:P0,f:V", "time=model", f"threads={threads}",
               f"warmup={warmup}", f"steps={steps}", "dump=0"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference driver failed: " + (r.stderr or r.stdout)[-400:])
        info = json.load(open(os.path.join(outd, "info.json")))
    return info["t_steps"], info


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "samples": len(sm), "reasons": sorted(reasons)}


def algorithmic_bytes(mesh, mf, nnz):
    """Bytes a value re-assembly must move at minimum (pattern cached):
    K values written, R written, u and f read, DOF map and vertex
    connectivity read, coordinates read, two per-element coefficients."""
    E, nb = mf.dofs.shape
    ndof = mf.nb_dof()
    return dict(K=8 * nnz, R=8 * ndof, u=8 * ndof, f=8 * ndof, dofmap=4 * nb * E,
                conn=4 * mesh.cvpts.shape[1] * E, coords=8 * mesh.points.size, coef=2 * 8 * E)


def cpu_time_oracle(nx, nthreads, reps=1):
    """One K + R assembly of the sub-mesh with the oracle; returns (seconds,
    elements)."""
    from oracle import gfref
    mesh, mf, mim, ws, data = make_problem(nx, seed=7)
    grp = ws.groups[0]
    slots = {d.slot: np.asarray(d.values, dtype=float) for d in ws.data.values() if d.slot >= 0}
    P2 = gfref.Problem(3, mesh.kind, 2, 3, mim.im, mesh.points, mesh.cvpts, mf.dofs, mf.nb_dof(),
                       grp.order2, slots)
    P1 = gfref.Problem(3, mesh.kind, 2, 3, mim.im, mesh.points, mesh.cvpts, mf.dofs, mf.nb_dof(),
                       grp.order1, slots)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        P2.matrix(nthreads)
        P1.vector(nthreads)
        ts.append(time.perf_counter() - t0)
    return min(ts), mesh.nb_convex()


def workload_config(nx, E, ndof, nnz):
    return {"workload": f"3-D P2 tet linear elasticity, regular_unit_mesh {nx}^3 x 6 tets, "
                        "IM_TETRAHEDRON(5), K + R value re-assembly, pattern cached",
            "elements": E, "n_dof": ndof, "nnz": nnz}


def run_reference(args, rank, world):
    """The reference arm: GetFEM's own multi-threaded model::assembly of the
    same workload (same mesh, seeds and expression) on all host cores."""
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    nx = args.nx
    E, ndof = 6 * nx ** 3, 3 * (2 * nx + 1) ** 3
    try:
        res = time_reference_model(nx, nthreads, args.warmup, args.steps)
    except RuntimeError as exc:
        res = None
        why = str(exc).splitlines()[-1] if str(exc) else "reference driver failed"
    else:
        why = "the reference build (oracle/_ref/ref_driver) is absent on this host"
    if res is None:
        print(json.dumps({"impl": "reference", "unavailable": why}), flush=True)
        return
    times, info = res
    mean_s = float(np.mean(times))
    v = E / mean_s
    sample = (f"GetFEM built from its sources with OpenMP, model::assembly(BUILD_ALL) "
              f"(K + right-hand side) of the full workload, {nthreads} threads, "
              f"nx={nx} ({E} elements) per step")
    cfg = workload_config(nx, E, ndof, int(info["nnz"]))
    cfg["l2"] = "host memory (CPU run)"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * mean_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded jittered mesh, lognormal coefficients, N(0,1) load)",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": "elements/s", "cores": nthreads,
                             "kind": "reference", "sample": sample},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_steps_s": times}
    print(json.dumps(line), flush=True)


def combine_ranks(dist, world, elements, ms, e2e_ms, device):
    """Replicas: every rank assembles its own copy of the workload.  The step
    time is the slowest rank's (max over ranks); the throughput counts the
    elements of all ranks over that time.  Returns (ms, e2e_ms, value, e2e)."""
    if dist is not None and world > 1:
        import torch
        tt = torch.tensor([ms, e2e_ms], device=device, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms, e2e_ms = float(tt[0]), float(tt[1])
    return ms, e2e_ms, world * elements / (ms * 1e-3), world * elements / (e2e_ms * 1e-3)


# ------------------------------------------------------- secondary workloads
# Each is measured after the headline line's timed region, on rank 0 of a
# one-GPU run, with CUDA events on the plans' stream (the default stream).

def _events_ms(fn, reps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_neohookean(steps, nx=32):
    """Q2 hexahedra 32^3 (32768 elements), compressible neo-Hookean, u = 8
    sinusoid modes of amplitude 0.05, per-element mu lognormal(0, 0.3): K + R
    (one pass) and the adjoint of the strain energy in mu and in the vertex
    coordinates (dE/du is R)."""
    import torch
    import getfem_gb300 as g
    from getfem_gb300 import _lib as L
    lib = L.lib()
    mesh = g.Mesh.regular_unit(3, nx, "hex")
    mf = g.MeshFem(mesh, 3, degree=2)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,5)")
    E = mesh.nb_convex()
    u, mu_np = neohookean_inputs(mf.basic_dof_nodes(), E)
    dev = "cuda"
    mu = torch.tensor(mu_np, device=dev)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=torch.tensor(u, device=dev))
    ws.add_fem_constant("mu", g.MeshFem(mesh, 1, degree=0), mu)
    ws.add_fixed_size_constant("D1", np.array([1.5]))
    ws.add_expression("Compressible_Neo_Hookean_potential(Grad_u,[0.5*mu;D1])", mim)
    grp = ws.groups[0]
    h1 = ws._plan(grp, grp.order1)
    ws._upload(h1, grp.order1, need_u=True)
    h0 = ws._plan(grp, grp.order0)
    ws._upload(h0, grp.order0, need_u=True)
    L.check(lib.gfgpu_assemble(h1, 2, L.WITH_VECTOR, None))
    gmu = torch.empty_like(mu)
    gX = torch.empty(mesh.points.size, dtype=torch.float64, device=dev)
    slot = ws.data["mu"].slot

    def kr():
        L.check(lib.gfgpu_assemble(h1, 2, L.WITH_VECTOR, None))

    def adj():
        L.check(lib.gfgpu_assemble(h0, 0, 0, None))
        L.check(lib.gfgpu_potential_gradient(h0, slot, C.c_void_p(gmu.data_ptr()), E, 1))
        L.check(lib.gfgpu_potential_gradient(h0, L.SLOT_POINTS, C.c_void_p(gX.data_ptr()),
                                             gX.numel(), 1))
    for _ in range(2):
        kr()
        adj()
    t_kr = _events_ms(kr, steps)
    t_adj = _events_ms(adj, steps)
    out = {"workload": f"Q2 hex {nx}^3 compressible neo-Hookean, IM_GAUSS_PARALLELEPIPED(3,5): "
                       "K + R, then energy + dE/dmu + dE/dX (dE/du = R)",
           "elements": E, "n_dof": mf.nb_dof(),
           "ms_K_R": t_kr, "ms_adjoint": t_adj,
           "elements_per_s_K_R": E / (t_kr * 1e-3),
           "elements_per_s_K_R_adjoint": E / ((t_kr + t_adj) * 1e-3)}
    del ws
    return out


def _batch_meshes(rng, n, lo, hi):
    """n (type, nx) pairs: element counts log-uniform in [lo, hi], types
    P1/P2 triangles (Poisson) and P1/P2 tetrahedra (elasticity)."""
    out = []
    for _ in range(n):
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        kind = int(rng.integers(4))
        if kind < 2:
            nx = max(2, int(round(np.sqrt(target / 2.0))))
        else:
            nx = max(2, int(round((target / 6.0) ** (1.0 / 3.0))))
        out.append((kind, nx))
    return out


def bench_batched(steps, n_meshes=512, lo=1e3, hi=2e5):
    """512 independent meshes, element counts log-uniform in [1e3, 2e5], a
    random mix of P1/P2 triangle Poisson and P1/P2 tetrahedron elasticity,
    coefficients lognormal(0, 0.2): K + R of every mesh, plain (one
    gfgpu_assemble per mesh) against batched (one persistent launch per
    kernel) and its CUDA graph replayed with coefficients perturbed in place.
    The same with many small meshes shows the launch-bound regime."""
    import gc
    import torch
    import getfem_gb300 as g
    from getfem_gb300 import _lib as L
    from getfem_gb300.batch import Batch
    lib = L.lib()
    rng = np.random.default_rng(4)
    dev = "cuda"
    t0 = time.perf_counter()
    wss = []
    plan_meshes = _batch_meshes(rng, n_meshes, lo, hi)
    # every coefficient field lives in one pool (a view per mesh), so that
    # the in-graph perturbation is one kernel
    sizes = []
    for kind, nx in plan_meshes:
        E = 2 * nx * nx if kind < 2 else 6 * nx ** 3
        sizes.append(E if kind < 2 else 2 * E)
    pool = torch.tensor(np.exp(rng.normal(0, 0.2, int(sum(sizes)))), device=dev)
    base = pool.clone()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    for (kind, nx), off in zip(plan_meshes, offs[:-1]):
        deg = 1 + kind % 2
        dim = 2 if kind < 2 else 3
        mesh = g.Mesh.regular_unit(dim, nx, "simplex")
        q = 1 if dim == 2 else 3
        mf = g.MeshFem(mesh, q, degree=deg)
        mf0 = g.MeshFem(mesh, 1, degree=0)
        E = mesh.nb_convex()
        ws = g.GaWorkspace()
        ws.add_fem_variable("u", mf, U=torch.tensor(rng.standard_normal(mf.nb_dof()) * 1e-2,
                                                    device=dev))
        assert E == (2 * nx * nx if dim == 2 else 6 * nx ** 3)
        if dim == 2:
            ws.add_fem_constant("kappa", mf0, pool[int(off):int(off) + E])
            ws.add_fem_constant("f", mf, torch.tensor(rng.uniform(-1, 1, mf.nb_dof()), device=dev))
            ws.add_expression("kappa*Grad_u.Grad_Test_u - f*Test_u",
                              g.MeshIm(mesh, "IM_TRIANGLE(2)" if deg == 1 else "IM_TRIANGLE(4)"))
        else:
            for k, nm in enumerate(("lambda", "mu")):
                ws.add_fem_constant(nm, mf0, pool[int(off) + k * E:int(off) + (k + 1) * E])
            ws.add_fem_constant("f", mf, torch.tensor(rng.standard_normal(mf.nb_dof()), device=dev))
            ws.add_expression(EXPR, g.MeshIm(mesh, "IM_TETRAHEDRON(2)" if deg == 1
                                             else "IM_TETRAHEDRON(5)"))
        wss.append(ws)
    b = Batch(wss)
    setup_s = time.perf_counter() - t0
    E_total = b.elements()
    grids = b.tune()
    plans = b.plans

    def plain():
        for h in plans:
            L.check(lib.gfgpu_assemble(h, 2, L.WITH_VECTOR, None))
    plain()
    t_plain = _events_ms(plain, max(1, steps // 4))
    t_batch = _events_ms(b.assemble, steps)
    factor = torch.ones(1, dtype=torch.float64, device=dev)

    def perturb():
        torch.mul(base, factor, out=pool)
    graph = b.graph(pre=perturb)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    torch.cuda.synchronize()
    e0.record()
    for r in range(reps):
        factor.fill_(1.0 + 0.01 * (r % 5))
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    b.sync()
    t_graph = e0.elapsed_time(e1) / reps
    out = {"workload": f"{n_meshes} meshes, element counts log-uniform in [{lo:g}, {hi:g}], "
                       "P1/P2 tri Poisson and P1/P2 tet elasticity, K + R per mesh",
           "meshes": n_meshes, "elements": int(E_total), "setup_s": setup_s,
           "grid_elem_pass": grids[0], "gather_launches": grids[1],
           "ms_plain": t_plain, "ms_batched": t_batch, "ms_graph_replay": t_graph,
           "elements_per_s_plain": E_total / (t_plain * 1e-3),
           "elements_per_s_batched": E_total / (t_batch * 1e-3),
           "elements_per_s_graph": E_total / (t_graph * 1e-3),
           "batched_over_plain": t_plain / t_batch, "graph_over_plain": t_plain / t_graph,
           "graph_replays": reps}
    del graph, b, wss, pool, base
    gc.collect()
    return out


def bench_q4(steps, nx=64):
    """Q4 hexahedra 64^3 (262144 elements, 16.97 M DOFs), per-element
    diffusivity lognormal(0, 0.5): assembled K + R, the matrix-free apply
    R = K u (order-1 assembly, no K), and the adjoint of u^T K u in the
    diffusivity (u i.i.d. N(0,1))."""
    import gc
    import torch
    import getfem_gb300 as g
    from getfem_gb300 import _lib as L
    lib = L.lib()
    t0 = time.perf_counter()
    mesh = g.Mesh.regular_unit(3, nx, "hex")
    mf = g.MeshFem(mesh, 1, degree=4)
    mim = g.MeshIm(mesh, "IM_GAUSS_PARALLELEPIPED(3,9)")
    E = mesh.nb_convex()
    dev = "cuda"
    kappa_np, u_np = q4_inputs(E, mf.nb_dof())
    kappa = torch.tensor(kappa_np, device=dev)
    u = torch.tensor(u_np, device=dev)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=u)
    ws.add_fem_constant("kappa", g.MeshFem(mesh, 1, degree=0), kappa)
    ws.add_expression("kappa*Grad_u.Grad_u", mim)
    grp = ws.groups[0]
    h1 = ws._plan(grp, grp.order1)
    ws._upload(h1, grp.order1, need_u=True)
    h0 = ws._plan(grp, grp.order0)
    ws._upload(h0, grp.order0, need_u=True)
    L.check(lib.gfgpu_assemble(h1, 2, L.WITH_VECTOR, None))
    L.check(lib.gfgpu_sync(h1))
    setup_s = time.perf_counter() - t0
    nr, nnz = C.c_int64(), C.c_int64()
    L.check(lib.gfgpu_pattern_size(h1, C.byref(nr), C.byref(nnz)))
    gk = torch.empty_like(kappa)
    slot = ws.data["kappa"].slot

    def kr():
        L.check(lib.gfgpu_assemble(h1, 2, L.WITH_VECTOR, None))

    def apply():
        L.check(lib.gfgpu_assemble(h1, 1, 0, None))

    def apply_sf():
        # opt-in: exact tensor-product basis, 1D contractions
        L.check(lib.gfgpu_assemble(h1, 1, L.SUM_FACTORISATION, None))

    def adj():
        L.check(lib.gfgpu_potential_gradient(h0, slot, C.c_void_p(gk.data_ptr()), E, 1))
    for f in (kr, apply, apply_sf, adj):
        f()
    t_kr = _events_ms(kr, steps)
    t_ap = _events_ms(apply, steps)
    t_adj = _events_ms(adj, steps)
    t_sf = _events_ms(apply_sf, steps)
    # deviation of the sum-factorised apply from the reference-exact one
    dvec = C.c_void_p()
    L.check(lib.gfgpu_device_vector(h1, C.byref(dvec)))
    n = mf.nb_dof()

    def vec_now():
        L.check(lib.gfgpu_sync(h1))
        v = torch.empty(n, dtype=torch.float64, device="cuda")
        L.check(lib.gfgpu_copy_result(h1, L.RESULT_VECTOR, C.c_void_p(v.data_ptr())))
        return v
    apply()
    r_ref = vec_now()
    apply_sf()
    r_sf = vec_now()
    scale = torch.maximum(r_ref.abs(), 1e-3 * r_ref.abs().max())
    sf_dev = float(((r_sf - r_ref).abs() / scale).max())
    out = {"workload": f"Q4 hex {nx}^3 kappa*Grad_u.Grad_Test_u, IM_GAUSS_PARALLELEPIPED(3,9): "
                       "K + R assembled, matrix-free R = K u, d(u^T K u)/dkappa",
           "elements": E, "n_dof": mf.nb_dof(), "nnz": nnz.value, "setup_s": setup_s,
           "ms_K_R": t_kr, "ms_matrix_free_apply": t_ap, "ms_adjoint_kappa": t_adj,
           "ms_matrix_free_apply_sum_factorised": t_sf,
           "sum_factorised_max_rel_deviation": sf_dev,
           "elements_per_s_K_R": E / (t_kr * 1e-3),
           "elements_per_s_apply": E / (t_ap * 1e-3),
           "elements_per_s_apply_sum_factorised": E / (t_sf * 1e-3),
           "elements_per_s_K_R_adjoint": E / ((t_kr + t_adj) * 1e-3)}
    del ws
    gc.collect()
    return out


def bench_poisson_cg():
    """64 x 64 P1 triangles, Grad_u.Grad_Test_u - f*Test_u, f U[-1,1],
    homogeneous Dirichlet on the boundary: assembly + elimination + CG to
    1e-12 (latency-bound: 4225 DOFs)."""
    import torch
    import getfem_gb300 as g
    from getfem_gb300 import solvers
    mesh = g.Mesh.regular_unit(2, 64, "simplex")
    mf = g.MeshFem(mesh, 1, degree=1)
    ws = g.GaWorkspace()
    ws.add_fem_variable("u", mf, U=np.zeros(mf.nb_dof()))
    ws.add_fem_constant("f", mf, poisson_inputs(mf.nb_dof()))
    ws.add_expression("Grad_u.Grad_Test_u - f*Test_u", g.MeshIm(mesh, "IM_TRIANGLE(2)"))
    dofs = solvers.boundary_dofs(mf)
    solvers.solve_linear(ws, dofs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u, info = solvers.solve_linear(ws, dofs)
    torch.cuda.synchronize()
    return {"workload": "64x64 P1 triangles Poisson, boundary Dirichlet, CG (identity) to 1e-12",
            "elements": mesh.nb_convex(), "n_dof": mf.nb_dof(),
            "ms_assemble_and_solve": 1e3 * (time.perf_counter() - t0),
            "cg_iterations": info["iterations"], "relative_residual": info["residual"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gfgpu", choices=["gfgpu", "reference"])
    ap.add_argument("--nx", type=int, default=40)
    ap.add_argument("--ref-nx", type=int, default=12)
    ap.add_argument("--cpu-nx", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-run", action="store_true",
                    help="short run for profilers: the timed steps and one profiled step only")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch configuration (no gfgpu_tune)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the secondary workloads (neo-Hookean, batched, Q4, CG)")
    ap.add_argument("--secondary", choices=["neohookean", "q4", "batched", "cg"],
                    help="run one secondary workload only (for profiling) and print it")
    ap.add_argument("--sec-nx", type=int, default=0,
                    help="mesh size of --secondary (default: the configuration's)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.secondary:
        import torch
        torch.cuda.set_device(local)
        nx = args.sec_nx
        fn = {"neohookean": lambda: bench_neohookean(args.steps, nx or 32),
              "q4": lambda: bench_q4(args.steps, nx or 64),
              "batched": lambda: bench_batched(args.steps),
              "cg": bench_poisson_cg}[args.secondary]
        print(json.dumps(fn()), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from getfem_gb300 import _lib as L
    lib = L.lib()
    mesh, mf, mim, ws, data = make_problem(args.nx)
    grp = ws.groups[0]
    h = ws._plan(grp, grp.order1)
    ws._upload(h, grp.order1, need_u=True)
    E = mesh.nb_convex()
    flags = L.WITH_VECTOR
    L.check(lib.gfgpu_assemble(h, 2, flags, None))  # builds the pattern
    L.check(lib.gfgpu_sync(h))
    nr, nnz = C.c_int64(), C.c_int64()
    L.check(lib.gfgpu_pattern_size(h, C.byref(nr), C.byref(nnz)))
    nnz = nnz.value
    # launch configuration: the autotuner's choice for this element family
    # (same bits for every candidate), picked before the warm-up
    launch = L.Launch()
    if args.no_tune:
        L.check(lib.gfgpu_get_launch(h, C.byref(launch)))
    else:
        L.check(lib.gfgpu_tune(h, 3, C.byref(launch)))
    for _ in range(args.warmup):
        L.check(lib.gfgpu_assemble(h, 2, flags, None))
    L.check(lib.gfgpu_sync(h))

    # device-resident timing (inputs, T scratch and K all exceed the 129 MB L2)
    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
    launches0 = lib.gfgpu_launch_count(h)
    sampler = ClockSampler(local)
    with sampler:
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            L.check(lib.gfgpu_assemble(h, 2, flags, None))
        e1.record()
        barrier()
    launches = lib.gfgpu_launch_count(h) - launches0
    L.check(lib.gfgpu_sync(h))
    ms = e0.elapsed_time(e1) / args.steps

    if args.profile_run:
        # a short run for profilers (ncu launch lists and captures): the
        # timed steps and one profiled step, nothing else
        L.check(lib.gfgpu_assemble(h, 2, flags | L.PROFILE, None))
        t = (C.c_float * 2)()
        L.check(lib.gfgpu_kernel_times(h, t, 2))
        L.check(lib.gfgpu_sync(h))
        if rank == 0:
            print(json.dumps({"profile_run": True, "workload": workload_config(args.nx, E, mf.nb_dof(), nnz),
                              "ms_per_step": ms, "kernels_ms": {"element_pass": t[0],
                                                                "row_gather": t[1]},
                              "launch": [launch.ep_threads, launch.gather_warps]}), flush=True)
        return

    # a longer run of the same step (about a second) with its own clock
    # record, for the steadiness of the figure above
    steady_steps = max(args.steps, 300)
    steady = ClockSampler(local)
    with steady:
        barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        for _ in range(steady_steps):
            L.check(lib.gfgpu_assemble(h, 2, flags, None))
        s1.record()
        barrier()
    steady_ms = s0.elapsed_time(s1) / steady_steps

    # per-kernel durations (CUDA events on the plan's stream)
    kt = np.zeros(2)
    nprof = min(args.steps, 20)
    for _ in range(nprof):
        L.check(lib.gfgpu_assemble(h, 2, flags | L.PROFILE, None))
        t = (C.c_float * 2)()
        L.check(lib.gfgpu_kernel_times(h, t, 2))
        kt += np.array([t[0], t[1]])
    kt /= nprof

    # end to end through the C ABI with pinned host buffers: u in, the
    # upper triangle of the symmetric K (gfgpu_assemble_host_upper; the
    # full K is its mirror, bit for bit) and R out every step; the same with
    # all nnz values (gfgpu_assemble_host) as a second figure
    u_h = torch.from_numpy(np.ascontiguousarray(data["u"])).pin_memory()
    vec_h = torch.empty(mf.nb_dof(), dtype=torch.float64).pin_memory()
    nnz_u = C.c_int64()
    L.check(lib.gfgpu_pattern_upper(h, C.byref(nnz_u), None, None))
    nnz_u = nnz_u.value
    # every call is synchronous (the values are in host memory when it
    # returns); the figure is the mean over the steps, and the per-call
    # median and maximum are reported beside it.  Single calls on the shared
    # host take tens of ms about every 0.5 s, so the loop runs about a second
    # (200 calls at the default step count) for the mean to hold them at
    # their long-run rate
    e2e_steps = max(50, min(2 * args.steps, 200))

    def host_loop(fn, out_h):
        for _ in range(3):
            L.check(fn(h, C.c_void_p(u_h.data_ptr()), C.c_void_p(out_h.data_ptr()),
                       C.c_void_p(vec_h.data_ptr())))
        barrier()
        calls = []
        import gc
        gc.disable()  # no collector pause inside the timed calls
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            tc = time.perf_counter()
            L.check(fn(h, C.c_void_p(u_h.data_ptr()), C.c_void_p(out_h.data_ptr()),
                       C.c_void_p(vec_h.data_ptr())))
            calls.append(1e3 * (time.perf_counter() - tc))
        t1 = time.perf_counter()
        gc.enable()
        barrier()
        return 1e3 * (t1 - t0) / e2e_steps, calls
    vals_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    e2e_full_ms, full_calls = host_loop(lib.gfgpu_assemble_host, vals_h)
    del vals_h
    uvals_h = torch.empty(nnz_u, dtype=torch.float64).pin_memory()
    e2e_ms, upper_calls = host_loop(lib.gfgpu_assemble_host_upper, uvals_h)
    del uvals_h

    ms, e2e_ms, value, e2e = combine_ranks(dist, world, E, ms, e2e_ms, "cuda")
    if rank != 0:
        dist.destroy_process_group()
        return

    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_source = ("MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                   else "6800 GB/s (of fallback: MEASURED_PEAKS.json absent)")
    ab = algorithmic_bytes(mesh, mf, nnz)
    step_bytes = sum(ab.values())
    # the dominant kernel of the step and its achieved rate on the step's
    # algorithmic bytes (pattern cached: K values and R written, inputs read)
    names = ["element_pass", "row_gather"]
    dom = int(np.argmax(kt))
    dom_gbs = step_bytes / (kt[dom] * 1e-3) / 1e9
    fp64_peak, dmma_peak, mixed_peak = C.c_double(), C.c_double(), C.c_double()
    L.check(lib.gfgpu_fp64_peak(0, C.byref(fp64_peak)))
    L.check(lib.gfgpu_fp64_peak(1, C.byref(dmma_peak)))
    L.check(lib.gfgpu_fp64_peak(2, C.byref(mixed_peak)))
    # FP64 flops the element pass executes per element (from its loop
    # structure): the node-pair blocks i <= j of the symmetric K_e (2 per
    # reference-tensor term per component pair), the load term, T (a multiply
    # and an FMA per upper entry, the c1 term on the diagonal blocks, 4
    # multiplies per row, |J| c1 g_v.g_w per vertex pair) and the geometry
    # (K u is formed by the row gather from the assembled rows)
    from getfem_gb300.tables import simplex_term_count, simplex_upper_term_count
    _, nb = simplex_term_count(3, 2)
    nterm_upper = simplex_upper_term_count(3, 2)
    qd, nv = 3, 4
    M = qd * nv
    s_ = nb * qd
    ep_flops = (2.0 * nterm_upper * qd * qd + 2.0 * s_ * nb
                + 3.0 * M * (M + 1) / 2 + qd * nv * (nv + 1) / 2 + 4.0 * M
                + 6.0 * nv * (nv + 1) / 2 + 90.0)
    ep_tflops = E * ep_flops / (kt[0] * 1e-3) / 1e12
    # DRAM bytes per launch of the dominant kernel: from one ncu capture of
    # the same kernel on the 20^3 x 6 mesh, scaled by the element count
    traffic = None
    fp64_ncu = None
    prof = os.path.join(ROOT, "profiles", "dram_bytes_per_element.json")
    if os.path.exists(prof):
        try:
            rec = _json.load(open(prof))
            traffic = float(rec[names[dom]]) * E
            fp64_ncu = rec.get("fp64_pipe_active", {}).get(names[dom])
        except (ValueError, TypeError, KeyError, AttributeError):
            traffic = None
    cpu = None
    if not args.no_cpu:
        nthreads = os.cpu_count() or 1
        res = None
        try:
            res = time_reference_model(args.nx, nthreads, 1, 3)
        except RuntimeError as exc:
            print(f"reference CPU baseline failed ({exc}); timing the oracle port", file=sys.stderr)
        if res is not None:
            tr = float(np.mean(res[0]))
            cpu = {"value": E / tr, "unit": "elements/s", "cores": nthreads, "kind": "reference",
                   "sample": f"GetFEM built from its sources with OpenMP, "
                             f"model::assembly(BUILD_ALL) of the full workload ({E} elements), "
                             f"{nthreads} threads, mean of 3 after 1 warm-up"}
        else:
            t, Es = cpu_time_oracle(args.cpu_nx, nthreads, reps=2)
            cpu = {"value": Es / t, "unit": "elements/s", "cores": nthreads, "kind": "port",
                   "sample": f"oracle (CPU restatement of the reference exec loop), OpenMP "
                             f"{nthreads} threads, K + R of the same problem at nx={args.cpu_nx} "
                             f"({Es} elements), best of 2"}
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded jittered mesh, lognormal coefficients, N(0,1) load)",
        "config": dict(workload_config(args.nx, E, mf.nb_dof(), nnz),
                       l2="inputs larger than L2 (K values, scratch and DOF data >> 129 MB)",
                       dofs_per_s=value * mf.nb_dof() / E,
                       launch={"ep_threads_per_element": launch.ep_threads,
                               "gather_warps_per_block": launch.gather_warps,
                               "autotuned": not args.no_tune}),
        "kernels_ms": {"element_pass": float(kt[0]), "row_gather": float(kt[1])},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": dom_gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": dom_gbs / hbm_peak,
                     "traffic": traffic, "algorithmic_bytes": step_bytes,
                     "peak_source": peak_source,
                     "fp64_pipe_active_ncu": fp64_ncu,
                     "limiter": "FP64 pipe and issue latency, not HBM: measured FP64 FMA "
                                f"{fp64_peak.value:.2f} TFLOP/s is 0.19 flop per HBM byte; "
                                "the fp64 object gives the element pass's FP64 fraction"},
        "fp64": {"kernel": "element_pass", "achieved_tflops": ep_tflops,
                 "peak_tflops": fp64_peak.value, "frac": ep_tflops / fp64_peak.value,
                 "flops_per_element": ep_flops,
                 "peak_source": "gfgpu_fp64_peak FMA microbenchmark, this run",
                 "dmma_peak_tflops": dmma_peak.value,
                 "fma_and_dmma_warps_tflops": mixed_peak.value},
        "steady": {"steps": steady_steps, "ms_per_step": steady_ms,
                   "elements_per_s": E / (steady_ms * 1e-3), "clocks": steady.summary()},
        "step_hbm_frac": step_bytes / (ms * 1e-3) / 1e9 / hbm_peak,
        "e2e": {"value": e2e, "unit": "elements/s", "h2d_bytes_per_step": 8 * mf.nb_dof(),
                "d2h_bytes_per_step": 8 * nnz_u + 8 * mf.nb_dof(), "ms_per_step": e2e_ms,
                "api": "gfgpu_assemble_host_upper (u in; the upper triangle of the "
                       "bit-symmetric K, nnz_upper values, and R out)", "nnz_upper": nnz_u,
                "steps": e2e_steps, "median_ms_per_call": float(np.median(upper_calls)),
                "max_ms_per_call": float(np.max(upper_calls))},
        "e2e_full_values": {"value": world * E / (e2e_full_ms * 1e-3), "unit": "elements/s",
                            "h2d_bytes_per_step": 8 * mf.nb_dof(),
                            "d2h_bytes_per_step": 8 * nnz + 8 * mf.nb_dof(),
                            "ms_per_step": e2e_full_ms, "api": "gfgpu_assemble_host",
                            "median_ms_per_call": float(np.median(full_calls)),
                            "max_ms_per_call": float(np.max(full_calls))},
        "gpu_launches": int(launches), "cpu_baseline": cpu, "clocks": sampler.summary(),
    }
    if not args.no_extra and world == 1:
        del ws
        import gc
        gc.collect()
        extra = {}
        for name, fn in (("poisson_cg", bench_poisson_cg),
                         ("neohookean_q2_hex", lambda: bench_neohookean(10)),
                         ("batched_512_meshes", lambda: bench_batched(10)),
                         ("batched_small_meshes", lambda: bench_batched(
                             10, n_meshes=4096, lo=1e2, hi=2e3)),
                         ("q4_hex_laplacian", lambda: bench_q4(5))):
            free0 = torch.cuda.mem_get_info()[0]
            try:
                extra[name] = fn()
            except Exception as exc:  # reported, not hidden
                extra[name] = {"error": f"{type(exc).__name__}: {exc}"}
            gc.collect()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            extra[name]["device_free_gb_before"] = free0 / 1e9
        line["secondary"] = extra
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
