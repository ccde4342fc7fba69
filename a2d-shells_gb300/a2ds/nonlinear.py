"""Nonlinear preload and buckling about the preloaded state.

The reference builds no Newton or continuation solver (TACSContinuation and
TACSIntegrator live only in its archive/); its building blocks are
TACSAssembler::assembleRes / assembleJacobian (src/TACSAssembler.cpp:4000,
4084), TACSSchurPc and the nonlinear shell elements
(TACSQuad4NonlinearShell, src/elements/shell/TACSShellElementDefs.h:27).
This module is the driver on top of the GB300 library:

* `newton_preload`: equal load increments s_k = load * k / nsteps; at each,
  full Newton on R(u) = s_k f with the exact tangent K_T(u) factored on the
  GPU each step (the C ABI's a2ds_newton_preload);
* `preload_buckling`: the eigenproblem K_T(u) x + lam G(u) x = 0 about the
  converged preload u, with G(u) the geometric stiffness along u (stated
  definition), solved by the library's shift-invert Lanczos;
* `preload_xpt_sens`: d(lam)/dX of one of those multipliers, the
  coordinate-sensitivity formula of the reference's (commented-out)
  TACSLinearBuckling::evalEigenXptSens (src/TACSBuckling.cpp:457-497) with
  the preload's Newton system K_T(u) in place of K: element states are
  recomputed from u and the coordinates on the GPU for every derivative
  (nothing of the Newton iterations is stored).
"""
from __future__ import annotations

import numpy as np

from . import capi


def _bc_mask_vector(assembler: capi.Assembler, bc_nodes, bc_mask):
    fixed = np.zeros((assembler.num_nodes, 6), bool)
    for node, mask in zip(np.asarray(bc_nodes), np.asarray(bc_mask)):
        for k in range(6):
            if int(mask) >> k & 1:
                fixed[node, k] = True
    return fixed


def newton_preload(assembler: capi.Assembler, rhs, bc_nodes=None, bc_mask=None, load: float = 1.0,
                   nsteps: int = 10, rtol: float = 1e-10, max_newton: int = 25,
                   precision: int = 64):
    """Newton load stepping to `load` times the nodal load vector `rhs`
    (node-major num_nodes x 6) on the GPU (a2ds_newton_preload; the
    Dirichlet set is the assembler's, bc_nodes / bc_mask are accepted for
    the caller's bookkeeping only).  Returns (u, iterations per step, final
    relative residual).  Raises A2dsError (A2DS_ERR_NOCONV) if a step does
    not converge."""
    import ctypes
    f = capi._f64(np.asarray(rhs, float).reshape(-1, 6))
    u = np.zeros_like(f)
    its = np.zeros(nsteps, np.int32)
    rel = ctypes.c_double()
    capi._check(assembler.lib.a2ds_newton_preload(
        assembler.h, capi._d(f), float(load), int(nsteps), float(rtol), int(max_newton),
        int(precision), capi._d(u), capi._i(its), ctypes.byref(rel)))
    return u, its.tolist(), rel.value


def preload_buckling(assembler: capi.Assembler, u, sigma: float, num_eigvals: int = 5,
                     max_lanczos: int = 120, eig_tol: float = 1e-10, precision: int = 64,
                     block_size: int = 4):
    """Lowest buckling multipliers about the preloaded state u:
    K_T(u) x + lam G(u) x = 0.  Returns (lam, LinearBuckling handle)."""
    KT, G = assembler.create_mat(), assembler.create_mat()
    assembler.assemble_jacobian(KT, u, want_res=False)
    assembler.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, u)
    b = capi.LinearBuckling(assembler, sigma, max_lanczos=max_lanczos, num_eigvals=num_eigvals,
                            eig_tol=eig_tol, precision=precision, block_size=block_size)
    lam = b.solve_matrices(KT, G)
    return lam, b, KT, G


def preload_xpt_sens(assembler: capi.Assembler, u, lam: float, phi, KT, G,
                     precision: int = 64, dh: float = 1e-7):
    """d(lam)/dX (num_nodes x 3) for K_T(u) phi + lam G(u) phi = 0 about the
    preload R(u, X) = s f (f fixed nodal loads):

      dlam/dX = -[phi^T K_T' phi + lam phi^T G' phi - psi^T R'] / (phi^T G phi),
      K_T(u) psi = d/du [phi^T (K_T(u) + lam G(u)) phi],

    ' = d/dX at fixed u.  KT and G are the matrices the buckling solve used
    (K_T(u) with its Dirichlet rows, G(u)).  All element derivatives are the
    library's element-by-element central differences (step dh)."""
    phi = np.asarray(phi, float).reshape(-1, 6)
    u = np.asarray(u, float).reshape(-1, 6)
    K_, G_ = capi.A2DS_STIFFNESS_MATRIX, capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX
    phiGphi = float(np.sum(phi * G.mult(phi)))
    if not np.isfinite(phiGphi) or phiGphi == 0.0:
        raise RuntimeError("phi^T G phi vanishes")
    g = (assembler.eval_mat_sv_sens_inner_product(K_, phi, phi, u, dh=dh)
         + lam * assembler.eval_mat_sv_sens_inner_product(G_, phi, phi, u, dh=dh))
    pc = capi.SchurPc(KT, 1000000, precision)
    pc.factor(KT)
    psi = pc.apply_factor(g)
    psi = psi + pc.apply_factor(g - KT.mult(psi))  # one refinement step
    dX = assembler.add_mat_xpt_sens_inner_product(1.0, K_, phi, phi, vars_=u, dh=dh)
    assembler.add_mat_xpt_sens_inner_product(lam, G_, phi, phi, dfdX=dX, vars_=u, dh=dh)
    assembler.add_adjoint_res_xpt_sens_products(-1.0, psi, dfdX=dX, vars_=u, dh=dh)
    return -dX / phiGphi
