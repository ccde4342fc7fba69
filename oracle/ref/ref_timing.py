"""Time the reference's own buckling solve (oracle/ref/cpu_ref_bench.cpp,
compiled from the reference's sources by oracle/ref/Makefile) beside the CPU
oracle's solve of the same cylinder on the same host threads.  Test
infrastructure: it calibrates the oracle port, which stands in for the
reference where the reference's sources cannot travel.

  python oracle/ref/ref_timing.py --nx 128 --ny 256 --threads 8 [--port] [--save F.npz]

--save writes the reference's loads with the workload and run details to an
npz fixture (tests/golden/cyl_q4_512x1024_ref_loads.npz came from
--nx 512 --ny 1024 --threads 8: 2.6 h on 8 x86 cores).

Only a machine with the reference sources builds cpu_ref_bench (the Makefile
reads them from REF, default the reference checkout beside this repository's
build environment; see the Makefile).  Prints one JSON line per run.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "a2d-shells_gb300"))
sys.path.insert(0, REPO)

from a2ds import mesh as meshgen  # noqa: E402

BIN = os.path.join(REPO, "oracle", "_ref", "cpu_ref_bench")


def write_inputs(d, m, sigma, lev, gm_m, gm_restarts, lanczos, nev, gm_tol, eig_tol, nreport):
    np.save(os.path.join(d, "X.npy"), np.ascontiguousarray(m.X, dtype=np.float64))
    np.save(os.path.join(d, "conn.npy"), np.ascontiguousarray(m.conn, dtype=np.int32))
    np.save(os.path.join(d, "bc_nodes.npy"), m.bc_nodes.astype(np.int32))
    np.save(os.path.join(d, "bc_mask.npy"), m.bc_mask.astype(np.int32))
    np.save(os.path.join(d, "bc_vals.npy"), np.ascontiguousarray(m.bc_vals, dtype=np.float64))
    np.save(os.path.join(d, "rhs.npy"), np.ascontiguousarray(m.rhs, dtype=np.float64))
    np.save(os.path.join(d, "elem_thickness.npy"), m.thickness.astype(np.float64))
    prm = np.array([m.E, m.nu, sigma, lev, gm_m, gm_restarts, lanczos, nev, 0,
                    gm_tol, 0.0, 0.0, eig_tol, nreport], dtype=np.float64)
    np.save(os.path.join(d, "params.npy"), prm)


def save_fixture(path, ref, nx, ny, vectors):
    """The reference run's loads and its set-up, as a test fixture."""
    np.savez(path, nx=nx, ny=ny, sigma=float(ref["sigma"]),
             eigvals=np.asarray(ref["eigvals"], np.float64),
             lanczos_vectors=vectors, threads=int(ref["threads"]),
             seconds=float(ref["seconds"]), gmres_iterations=int(ref["gmres_iterations"]),
             gmres_cycles=int(ref["gmres_cycles"]))


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--nx", type=int, default=128)
    p.add_argument("--ny", type=int, default=256)
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    p.add_argument("--neig", type=int, default=10, help="loads reported")
    p.add_argument("--vectors", type=int, default=76,
                   help="Lanczos vectors of the reference: its num_eigvals, since its "
                        "Lanczos stops at num_eigvals vectors (default: the GPU solve's "
                        "count on the 512x1024 cylinder)")
    p.add_argument("--gmres", type=int, nargs=2, default=[10, 15],
                   help="GMRES subspace size and restarts (the cylinder example's)")
    p.add_argument("--gmres-tol", type=float, default=1e-12)
    p.add_argument("--eig-tol", type=float, default=1e-8)
    p.add_argument("--port", action="store_true",
                   help="also time the CPU oracle's solve on the same threads")
    p.add_argument("--save", help="write the reference's loads to this npz fixture")
    args = p.parse_args(argv)
    if not os.path.exists(BIN):
        print(json.dumps({"unavailable": "oracle/_ref/cpu_ref_bench is not built "
                                         "(make -C oracle/ref needs the reference sources)"}))
        return 0
    m = meshgen.cylinder(args.nx, args.ny)
    # the same shift as the benchmark's solves: 0.35 x the classical load
    sigma = 0.35 * meshgen.classical_cylinder_load(m.E, m.nu, m.meta["t"], 1.0)
    with tempfile.TemporaryDirectory() as d:
        write_inputs(d, m, sigma, 1000000, args.gmres[0], args.gmres[1], args.vectors + 1,
                     args.vectors, args.gmres_tol, args.eig_tol, args.neig)
        # OpenBLAS (the reference's BLAS here) single-threaded: its own threads
        # spin inside every small vector operation of GMRES
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        r = subprocess.run([BIN, d, str(args.threads)], capture_output=True, text=True,
                           check=True, env=env)
    line = next(ln for ln in r.stdout.splitlines() if ln.startswith("{"))
    ref = json.loads(line)
    ref.update(kind="reference", workload=f"cylinder {args.nx}x{args.ny}", sigma=sigma)
    print(json.dumps(ref), flush=True)
    if args.save:
        save_fixture(args.save, ref, args.nx, args.ny, args.vectors)
    if args.port:
        os.environ["OMP_NUM_THREADS"] = str(args.threads)
        import oracle
        t0 = time.perf_counter()
        plan = oracle.CpuPlan(m)
        t_plan = time.perf_counter() - t0
        t0 = time.perf_counter()
        lam, t, nvec = oracle.cpu_buckling_solve(m, plan, sigma, neig=args.neig, block=4,
                                                 eig_tol=args.eig_tol)
        secs = time.perf_counter() - t0
        rel = float(np.max(np.abs(np.sort(lam) - np.sort(ref["eigvals"])) /
                           np.abs(np.sort(ref["eigvals"]))))
        print(json.dumps({"kind": "port", "workload": f"cylinder {args.nx}x{args.ny}",
                          "threads": plan.threads, "seconds": secs, "setup_s": t_plan,
                          "phases_s": {k: round(v, 3) for k, v in t.items()},
                          "lanczos_vectors": int(nvec), "factor_blocks": int(plan.fcols.size),
                          "eigvals": [float(x) for x in lam],
                          "max_rel_diff_vs_reference": rel}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
