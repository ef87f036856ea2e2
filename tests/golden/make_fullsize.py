"""Generates the full-size golden fixtures tests/golden/full_*.npz from the
reference GetFEM build (oracle/_ref/ref_driver, made by
`make -C oracle/refbuild`), on the exact inputs of the benchmark workloads
(the seeded generators of bench.py).

The reference runs its own ga_workspace (add_expression + assembly(2) and
assembly(1), src/getfem_generic_assembly_workspace.cc:545, :791) on the
configurations at their full sizes:

  full_p1tri_poisson_64     64 x 64 P1 triangles, Grad_u.Grad_Test_u - f*Test_u
  full_p2tet_elastic_40     40^3 x 6 P2 tetrahedra, jittered, isotropic elasticity
                            with per-element lambda, mu and a nodal load
  full_q2hex_neohookean_32  32^3 Q2 hexahedra, the neo-Hookean brick form at
                            the 8-mode sinusoid displacement
  full_q4hex_laplace_8      8^3 Q4 hexahedra (a sub-mesh of the 64^3
                            workload), kappa*Grad_u.Grad_Test_u

A CSR of 1e8 entries is too large to commit, so each fixture keeps what a
comparison needs and stays small: nnz and the SHA-256 of the row pointers
and column indices (as little-endian int64), every entry of a few hundred
seeded rows, a few thousand seeded single entries, R at seeded positions
(all of R when it is small) with its maximum, and bilinear probes
w^T K v and w . R with seeded vectors w, v (regenerated from their seed by
the tests) together with the sums of |w_i K_ij v_j| that scale their
tolerance: every entry of K enters a probe.  The 64 x 64 case keeps K and
R whole.

Run from the repository root:  python tests/golden/make_fullsize.py [names]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NH = "((Id(meshdim)+Grad_u)*(Compressible_Neo_Hookean_PK2(Grad_u,[0.5*mu;D1]))):Grad_Test_u"
ELAST = "(lambda*Div_u*Id(3)+2*mu*Sym(Grad_u)):Grad_Test_u - f.Test_u"

N_ROWS = 400        # rows kept whole (at most)
N_ROW_ENTRIES = 40_000
N_ENTRIES = 4096    # single entries
N_RVALS = 8192      # R values (when R is not kept whole)
N_PROBES = 4        # bilinear probes
PROBE_SEED = 77
WHOLE_LIMIT = 200_000  # keep K and R whole below this many nonzeros


def sha256_i64(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def sha256_f8(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def probe_vectors(n: int, k: int, seed: int = PROBE_SEED):
    """The probe vectors w_k, v_k (N(0,1)), regenerated by the tests."""
    rng = np.random.default_rng(seed)
    return [(rng.standard_normal(n), rng.standard_normal(n)) for _ in range(k)]


def compact_record(rowptr, colidx, vals, R, seed):
    """The fixture fields of an assembled K (CSR, int64 indices) and R."""
    n = rowptr.size - 1
    nnz = int(rowptr[-1])
    rec = {"nnz": np.array([nnz]), "n_rows": np.array([n]),
           "rowptr_sha256": np.array(sha256_i64(rowptr)),
           "colidx_sha256": np.array(sha256_i64(colidx)),
           "R_max": np.array([np.abs(R).max()])}
    if nnz <= WHOLE_LIMIT:
        rec.update(K_rowptr=rowptr, K_colidx=colidx.astype(np.int32), K_vals=vals, R=R)
    else:
        rng = np.random.default_rng(seed)
        # about N_ROW_ENTRIES entries in the whole rows kept
        nrows = int(min(N_ROWS, max(50, N_ROW_ENTRIES * n // nnz)))
        rows = np.sort(rng.choice(n, nrows, replace=False))
        lens = rowptr[rows + 1] - rowptr[rows]
        rptr = np.concatenate([[0], np.cumsum(lens)])
        sel = np.concatenate([np.arange(rowptr[r], rowptr[r + 1]) for r in rows])
        pos = np.sort(rng.choice(nnz, N_ENTRIES, replace=False))
        ent_row = np.searchsorted(rowptr, pos, side="right") - 1
        ridx = np.sort(rng.choice(n, N_RVALS, replace=False))
        rec.update(rows=rows, rows_ptr=rptr, rows_col=colidx[sel].astype(np.int32),
                   rows_val=vals[sel], ent_row=ent_row, ent_col=colidx[pos].astype(np.int32),
                   ent_val=vals[pos], R_idx=ridx, R_val=R[ridx])
    # bilinear probes: w^T K v and w . R, each with the sum of the absolute
    # products that scales its tolerance
    row_of = np.repeat(np.arange(n), np.diff(rowptr))
    wkv, wkv_abs, wr, wr_abs = [], [], [], []
    for w, v in probe_vectors(n, N_PROBES):
        t = w[row_of] * vals * v[colidx]
        wkv.append(t.sum())
        wkv_abs.append(np.abs(t).sum())
        wr.append(w @ R)
        wr_abs.append(np.abs(w * R).sum())
    rec.update(probe_wKv=np.array(wkv), probe_wKv_abs=np.array(wkv_abs),
               probe_wR=np.array(wr), probe_wR_abs=np.array(wr_abs))
    return rec


def run_reference(dim, nx, gt, deg, qdim, im, expr, inputs, consts, jitter=None):
    """Runs ref_driver (orders 2 then 1) and returns (rowptr, colidx, vals,
    R, info)."""
    with tempfile.TemporaryDirectory() as td:
        ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        for k, v in inputs.items():
            np.asarray(v, dtype=np.float64).tofile(os.path.join(ind, k + ".bin"))
        if jitter is not None:
            jitter.astype(np.float64).tofile(os.path.join(ind, "jitter.bin"))
        cs = ",".join(f"{k}:{v}" for k, v in consts.items())
        cmd = [DRIVER, f"dim={dim}", f"nx={nx}", f"gt={gt}", f"fem={deg}", f"qdim={qdim}",
               f"im={im}", f"in={ind}", f"out={outd}", f"expr={expr}", "orders=2,1",
               f"jitter={1 if jitter is not None else 0}", f"consts={cs}", "dump=0"]
        subprocess.run(cmd, check=True)
        info = json.load(open(os.path.join(outd, "info.json")))

        def rd(fn, dt=np.float64):
            return np.fromfile(os.path.join(outd, fn), dtype=dt)
        return (rd("K_rowptr.bin", np.int64), rd("K_colidx.bin", np.int64), rd("K_vals.bin"),
                rd("R.bin"), info)


def case_inputs(name):
    """(driver args, inputs, consts, jitter, meta) of a full-size case, from
    the benchmark's own generators."""
    import bench
    if name == "full_p1tri_poisson_64":
        nx = 64
        ndof = (nx + 1) ** 2
        return (dict(dim=2, nx=nx, gt="PK", deg=1, qdim=1, im="IM_TRIANGLE(2)",
                     expr="Grad_u.Grad_Test_u - f*Test_u"),
                {"u": np.zeros(ndof), "f": bench.poisson_inputs(ndof)}, {"f": "V"}, None,
                {"generator": "bench.poisson_inputs(ndof, seed=1)"})
    if name == "full_p2tet_elastic_40":
        nx = 40
        jit, d = bench.p2tet_inputs(nx)
        return (dict(dim=3, nx=nx, gt="PK", deg=2, qdim=3, im="IM_TETRAHEDRON(5)", expr=ELAST),
                {"u": d["u"], "lambda": d["lam"], "mu": d["mu"], "f": d["f"]},
                {"lambda": "P0", "mu": "P0", "f": "V"}, jit,
                {"generator": "bench.p2tet_inputs(40, seed=2026)"})
    if name == "full_q2hex_neohookean_32":
        import getfem_gb300 as g
        nx = 32
        mesh = g.Mesh.regular_unit(3, nx, "hex")
        mf = g.MeshFem(mesh, 3, degree=2)
        u, mu = bench.neohookean_inputs(mf.basic_dof_nodes(), mesh.nb_convex())
        return (dict(dim=3, nx=nx, gt="QK", deg=2, qdim=3, im="IM_GAUSS_PARALLELEPIPED(3,5)",
                     expr=NH),
                {"u": u, "mu": mu, "D1": np.array([1.5])}, {"mu": "P0", "D1": "C"}, None,
                {"generator": "bench.neohookean_inputs(dof nodes, E, seed=3), D1 = 1.5"})
    if name == "full_q4hex_laplace_8":
        nx = 8
        E, ndof = nx ** 3, (4 * nx + 1) ** 3
        kappa, u = bench.q4_inputs(E, ndof)
        return (dict(dim=3, nx=nx, gt="QK", deg=4, qdim=1, im="IM_GAUSS_PARALLELEPIPED(3,9)",
                     expr="kappa*Grad_u.Grad_Test_u"),
                {"u": u, "kappa": kappa}, {"kappa": "P0"}, None,
                {"generator": "bench.q4_inputs(E, ndof, seed=5) at nx=8"})
    raise KeyError(name)


NAMES = ["full_p1tri_poisson_64", "full_p2tet_elastic_40", "full_q2hex_neohookean_32",
         "full_q4hex_laplace_8"]


def make(name, seed):
    args, inputs, consts, jit, meta = case_inputs(name)
    t0 = time.time()
    rowptr, colidx, vals, R, info = run_reference(args["dim"], args["nx"], args["gt"],
                                                  args["deg"], args["qdim"], args["im"],
                                                  args["expr"], inputs, consts, jit)
    rec = compact_record(rowptr, colidx, vals, R, seed)
    # the generated inputs, so that a host whose generator gives other bits
    # is told so before any value is compared
    hashes = {k: sha256_f8(v) for k, v in inputs.items()}
    if jit is not None:
        hashes["jitter"] = sha256_f8(jit)
    meta.update(input_sha256=hashes)
    meta.update(name=name, dim=args["dim"], nx=args["nx"], gt=args["gt"], degree=args["deg"],
                qdim=args["qdim"], im=args["im"], expr=args["expr"], consts=consts,
                n_dof=info["n_dof"], n_elements=info["n_elements"], nnz=info["nnz"],
                sample_seed=seed, probe_seed=PROBE_SEED,
                reference_seconds={"assembly(2)": info.get("t_order2"),
                                   "assembly(1)": info.get("t_order1"),
                                   "host": "x86-64, 1 thread, GetFEM built from its sources"})
    rec["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "ndof", info["n_dof"], "nnz", info["nnz"], f"{time.time() - t0:.1f} s",
          flush=True)


def main():
    if not os.path.exists(DRIVER):
        sys.exit(f"{DRIVER} missing: build it with make -C oracle/refbuild")
    only = set(sys.argv[1:])
    for i, name in enumerate(NAMES):
        if not only or name in only:
            make(name, 3000 + i)


if __name__ == "__main__":
    main()
