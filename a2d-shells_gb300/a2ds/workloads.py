"""The named workloads beyond the benchmark's linear solve, run end to end
through the library and reported as one JSON line each.

  preload   buckling about a nonlinear preloaded state of the imperfect
            cylinder (0.1 t imperfection, Quad4 nonlinear shells): Newton
            load stepping to half the linear critical load in equal
            increments with the exact tangent (a2ds_newton_preload), the
            lowest loads of K_T(u) x + lambda G(u) x = 0
            (a2ds_preload_buckling), dlambda_1/ds_p for the 64 radial
            shape parameters (a2ds_preload_xpt_sens contracted with dX/ds_p)
            and central differences of whole Newton + buckling solves on
            seeded parameters;
  panel     the stiffened panel (Quad9 skin and blade webs, 400 thickness
            groups): lowest loads and dlambda/dt_g for every group, with
            central differences of whole solves on seeded groups.

Usage: python -m a2ds.workloads preload [--nx 256 --ny 512 ...]
       python -m a2ds.workloads panel [--nx 1360 --ny 408 --nz 41 ...]
The reference has the building blocks of both (assembleRes /
assembleJacobian, TACSSchurPc, the nonlinear and Quad9 shell elements) but no
driver for them.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import capi
from . import mesh as meshgen


def _assembler(m, X=None, nonlinear=False, tvals=None, groups=None):
    a = capi.Assembler(m.X if X is None else X, m.conn, nonlinear=nonlinear)
    a.set_material(m.E, m.nu)
    if tvals is None:
        a.set_thickness([m.meta["t"]])
    else:
        a.set_thickness(np.asarray(tvals, float), groups)
    a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    return a


def run_preload(args):
    m = meshgen.cylinder(args.nx, args.ny, imperfection=0.1)
    t = m.meta["t"]
    out = {"workload": f"preload: cylinder {args.nx}x{args.ny} Quad4 nonlinear shells, "
                       f"imperfection 0.1 t, {args.increments} Newton increments to "
                       f"{args.fraction} x the linear critical load, {args.neig} loads about "
                       f"the deformed state, 64 shape parameters",
           "dof": 6 * m.num_nodes, "precision": args.precision}
    lam_cl = meshgen.classical_cylinder_load(m.E, m.nu, t, 1.0)
    # linear critical load of the same (imperfect) cylinder
    t0 = time.perf_counter()
    a_lin = _assembler(m)
    b = capi.LinearBuckling(a_lin, 0.35 * lam_cl, max_lanczos=200, num_eigvals=1, eig_tol=1e-10,
                            precision=args.precision, block_size=4)
    lam_lin = float(b.solve(m.rhs, want_vectors=False)[0])
    out["linear_critical_load"] = lam_lin
    out["linear_solve_s"] = time.perf_counter() - t0
    del a_lin, b
    load = args.fraction * lam_lin

    def preload_solve(X, want_sens=False):
        a = _assembler(m, X=X, nonlinear=True)
        ts = time.perf_counter()
        its = np.zeros(args.increments, np.int32)
        u = np.zeros((m.num_nodes, 6))
        import ctypes
        rel = ctypes.c_double()
        capi._check(a.lib.a2ds_newton_preload(
            a.h, capi._d(capi._f64(m.rhs)), float(load), int(args.increments), 1e-10, 25,
            int(args.precision), capi._d(u), capi._i(its), ctypes.byref(rel)))
        t_newton = time.perf_counter() - ts
        ts = time.perf_counter()
        bb = capi.LinearBuckling(a, args.sigma_frac * (1.0 - args.fraction) / args.fraction,
                                 max_lanczos=200, num_eigvals=args.neig, eig_tol=1e-10,
                                 precision=args.precision, block_size=4)
        lam = bb.solve_preloaded(u, want_vectors=False).copy()
        t_buck = time.perf_counter() - ts
        res = {"lam": lam, "newton_iters": its.tolist(), "newton_rel": rel.value,
               "newton_s": t_newton, "buckling_s": t_buck}
        if want_sens:
            ts = time.perf_counter()
            res["dX"] = bb.eval_preload_xpt_sens(0)
            res["sens_s"] = time.perf_counter() - ts
        return res

    base = preload_solve(m.X, want_sens=True)
    modes = meshgen.radial_shape_modes(m)
    ds = np.array([float(np.sum(base["dX"] * modes[p])) for p in range(modes.shape[0])])
    out.update({"eigvals": base["lam"].tolist(), "newton_iters": base["newton_iters"],
                "newton_rel": base["newton_rel"], "newton_s": base["newton_s"],
                "buckling_s": base["buckling_s"], "shape_sens_s": base["sens_s"],
                "dlam1_ds": ds.tolist()})
    # central differences of whole solves on seeded parameters among those
    # with a first-order effect: on the (nearly) axisymmetric cylinder a
    # non-axisymmetric shape mode (n > 0) changes lambda_1 at second order
    # only (a rotation by pi / n maps +s to -s), so its derivative is zero up
    # to the imperfection and both the adjoint and the difference quotient
    # show their noise floors there
    fd = []
    rng = np.random.default_rng(meshgen.DEFAULT_SEED)
    mag = np.abs(ds)
    significant = np.where(mag >= 1e-3 * mag.max())[0]
    out["fd_candidates"] = significant.tolist()
    gap = abs(base["lam"][1] - base["lam"][0])
    for p in rng.choice(significant, min(args.fd_params, significant.size), replace=False):
        # the step moves lambda_1 by 1 % of its gap to lambda_2 at most, so
        # the difference quotient does not cross into the next eigenvalue
        eps = min(args.fd_step, 0.01 * gap / max(abs(ds[p]), 1e-300))
        lp = preload_solve(m.X + eps * modes[p])["lam"][0]
        lm = preload_solve(m.X - eps * modes[p])["lam"][0]
        d = (lp - lm) / (2 * eps)
        fd.append({"param": int(p), "step": eps, "adjoint": ds[p], "central_difference": d,
                   "rel_diff": abs(ds[p] - d) / max(abs(d), 1e-300),
                   "diff_vs_gradient_max": abs(ds[p] - d) / mag.max()})
    out["fd_check"] = fd
    out["lam_gap_rel"] = float(abs(base["lam"][1] - base["lam"][0]) / abs(base["lam"][0]))
    return out


def run_panel(args):
    ts = time.perf_counter()
    m = meshgen.stiffened_panel(args.nx, args.ny, args.nz)
    tv = m.meta["tvals"]
    a = _assembler(m, tvals=tv, groups=m.dv_group)
    out = {"workload": f"stiffened panel {args.nx}x{args.ny}x{args.nz} Quad9, "
                       f"{m.num_elements} elements, 400 thickness groups",
           "dof": 6 * m.num_nodes, "precision": args.precision,
           "setup_s": time.perf_counter() - ts}

    # shift: 0.9 x the lowest load of a cheap first solve about a small shift
    # (the loads of smallest magnitude converge first either way)
    # complete LU: a level of fill at least the node count (the panel has
    # more than the reference's customary lev = 1e6 nodes)
    lev = max(1000000, m.num_nodes)
    b0 = capi.LinearBuckling(a, args.sigma, max_lanczos=200, num_eigvals=1, eig_tol=1e-6,
                             lev_fill=lev, precision=args.precision, block_size=4)
    try:
        b0.solve(m.rhs, want_vectors=False)
    except capi.A2dsError:
        pass
    sigma = 0.9 * float(b0.eigvals[0])
    out["sigma"] = sigma
    out["first_solve_s"] = time.perf_counter() - ts
    del b0

    def solve(aa):
        bb = capi.LinearBuckling(aa, sigma, max_lanczos=200, num_eigvals=args.neig,
                                 eig_tol=1e-10, lev_fill=lev, precision=args.precision,
                                 block_size=4)
        lam = bb.solve(m.rhs, want_vectors=False).copy()
        return bb, lam

    ts = time.perf_counter()
    b, lam = solve(a)
    out["solve_s"] = time.perf_counter() - ts
    out["stats"] = b.stats()
    out["eigvals"] = lam.tolist()
    ts = time.perf_counter()
    d = b.eig_sens_thickness(0, tv.size)
    out["sens_s"] = time.perf_counter() - ts
    out["dlam1_dt"] = d.tolist()
    fd = []
    used = np.unique(m.dv_group)
    rng = np.random.default_rng(meshgen.DEFAULT_SEED)
    for g in rng.choice(used, args.fd_groups, replace=False):
        h = 1e-6 * tv[g]
        vals = []
        for sgn in (1.0, -1.0):
            t2 = tv.copy()
            t2[g] += sgn * h
            a.set_thickness(t2, m.dv_group)
            vals.append(solve(a)[1][0])
        a.set_thickness(tv, m.dv_group)
        c = (vals[0] - vals[1]) / (2 * h)
        fd.append({"group": int(g), "adjoint": float(d[g]), "central_difference": float(c),
                   "rel_diff": float(abs(d[g] - c) / max(abs(c), 1e-300))})
    out["fd_check"] = fd
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("workload", choices=["preload", "panel"])
    p.add_argument("--nx", type=int)
    p.add_argument("--ny", type=int)
    p.add_argument("--nz", type=int, default=41)
    p.add_argument("--precision", type=int, default=64, choices=[64, 48, 32])
    p.add_argument("--neig", type=int, default=5)
    p.add_argument("--increments", type=int, default=10)
    p.add_argument("--fraction", type=float, default=0.5)
    p.add_argument("--sigma-frac", type=float, default=0.9,
                   help="preload: shift = sigma_frac x (1 - fraction) / fraction, the "
                        "expected multiplier of the remaining load")
    p.add_argument("--sigma", type=float, default=100.0,
                   help="panel: shift of the first solve that fixes the shift")
    p.add_argument("--fd-params", type=int, default=4)
    p.add_argument("--fd-step", type=float, default=1e-5)
    p.add_argument("--fd-groups", type=int, default=10)
    args = p.parse_args(argv)
    capi.load()
    if args.workload == "preload":
        args.nx, args.ny = args.nx or 256, args.ny or 512
        out = run_preload(args)
    else:
        args.nx, args.ny = args.nx or 1360, args.ny or 408
        out = run_panel(args)
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
