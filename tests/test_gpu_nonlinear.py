"""Buckling about a nonlinear preloaded state (the nonlinear-preload row of
the scope: Newton load stepping on the nonlinear shell model with the exact
tangent, then K_T(u) x + lam G(u) x = 0).  Equilibrium of the GPU Newton
solution is checked with the CPU oracle's element residuals (restated from
TACSShellElement::addResidual with the nonlinear strain model); the
eigenvalues against a dense FP64 eigensolve of the same matrices."""
import numpy as np
import pytest

import oracle
from a2ds import capi
from a2ds import mesh as meshgen
from a2ds import nonlinear


def cpu_residual(m, u, t):
    """Assembled nonlinear residual R(u) from the oracle's element residuals."""
    mat = oracle.Material.iso(m.E, m.nu, t)
    R = np.zeros((m.num_nodes, 6))
    for e in range(m.num_elements):
        nodes = m.conn[e]
        re = oracle.element_residual(2, 1, mat, m.X[nodes], u[nodes].ravel())
        R[nodes] += re.reshape(-1, 6)
    return R


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 48])
def test_newton_preload_and_buckling(precision):
    m = meshgen.cylinder(8, 16)
    t = m.meta["t"]
    a = capi.Assembler(m.X, m.conn, nonlinear=True)
    a.set_material(m.E, m.nu)
    a.set_thickness([t])
    a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    load = 0.3 * meshgen.classical_cylinder_load(m.E, m.nu, t, 1.0)
    u, its, rel = nonlinear.newton_preload(a, m.rhs, m.bc_nodes, m.bc_mask, load, nsteps=4,
                                           rtol=1e-10, precision=precision)
    assert rel <= 1e-10
    assert max(its) <= 8, its  # Newton with the exact tangent converges fast
    # equilibrium on the free DOFs, by the CPU restatement of the element residual
    fixed = nonlinear._bc_mask_vector(a, m.bc_nodes, m.bc_mask)
    f = load * m.rhs
    R = cpu_residual(m, u, t)
    r = (R - f)[~fixed]
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(f[~fixed])
    assert np.abs(u[fixed]).max() == 0.0
    # buckling about the preloaded state
    KT, G = a.create_mat(), a.create_mat()
    a.assemble_jacobian(KT, u, want_res=False)
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, u)
    from test_gpu_solve import dense_buckling
    dense = dense_buckling(KT.to_dense_nodes(), G.to_dense_nodes(), m.bc_nodes, m.bc_mask)
    nev = 4
    lam, b, _, _ = nonlinear.preload_buckling(a, u, 0.95 * dense[0], num_eigvals=nev,
                                              eig_tol=1e-12, precision=precision, block_size=4)
    assert np.max(np.abs(lam - dense[:nev]) / np.abs(dense[:nev])) < 1e-8, (lam, dense[:nev])


@pytest.mark.gpu
def test_preload_buckling_xpt_sensitivity_vs_finite_difference():
    """d(lam)/dX about a nonlinear preloaded state (nonlinear.preload_xpt_sens:
    the evalEigenXptSens formula with the Newton tangent K_T(u) in the load-path
    adjoint and element states recomputed on the GPU) contracted with
    axisymmetric radial shape modes, against central differences of whole
    Newton + buckling solves on the moved meshes; rigid translations and
    rotations about the axis leave the multiplier unchanged."""
    m = meshgen.cylinder(8, 16)
    t = m.meta["t"]
    load = 0.3 * meshgen.classical_cylinder_load(m.E, m.nu, t, 1.0)
    modes = meshgen.radial_shape_modes(m)
    sigma = None

    def solve(X):
        nonlocal sigma
        a = capi.Assembler(X, m.conn, nonlinear=True)
        a.set_material(m.E, m.nu)
        a.set_thickness([t])
        a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
        a.initialize(capi.A2DS_TACS_AMD_ORDER)
        u, _, _ = nonlinear.newton_preload(a, m.rhs, m.bc_nodes, m.bc_mask, load, nsteps=4,
                                           rtol=1e-11)
        if sigma is None:
            from test_gpu_solve import dense_buckling
            KT, G = a.create_mat(), a.create_mat()
            a.assemble_jacobian(KT, u, want_res=False)
            a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, u)
            sigma = 0.95 * dense_buckling(KT.to_dense_nodes(), G.to_dense_nodes(), m.bc_nodes,
                                          m.bc_mask)[0]
        lam, b, KT, G = nonlinear.preload_buckling(a, u, sigma, num_eigvals=2, eig_tol=1e-12,
                                                   block_size=2)
        return a, u, lam, b, KT, G

    a, u, lam, b, KT, G = solve(m.X)
    dX = nonlinear.preload_xpt_sens(a, u, lam[0], b.eigvecs[0], KT, G)
    assert dX.shape == m.X.shape and np.all(np.isfinite(dX))
    scale = np.abs(dX).sum()
    assert np.all(np.abs(dX.sum(axis=0)) <= 1e-5 * scale), dX.sum(axis=0)
    spin = np.stack([np.zeros(m.num_nodes), -m.X[:, 2], m.X[:, 1]], axis=1)
    assert abs(np.sum(dX * spin)) <= 1e-5 * scale
    eps = 1e-4
    for p in (0, 8):  # (m, n) = (1, 0), (2, 0)
        ds = float(np.sum(dX * modes[p]))
        fd = (solve(m.X + eps * modes[p])[2][0] - solve(m.X - eps * modes[p])[2][0]) / (2 * eps)
        assert abs(ds - fd) <= 1e-4 * abs(fd), (p, ds, fd)


@pytest.mark.gpu
def test_preload_c_entries_match_composition():
    """The C ABI's preload entries (a2ds_preload_buckling and
    a2ds_preload_xpt_sens, reachable from C++ callers) against the same
    formula composed from the element-level entries in a2ds.nonlinear, on a
    cylinder with a large imperfection so that the lowest multiplier is
    simple (for a double one each solve may return another eigenvector of
    the pair, and the coordinate derivative depends on it)."""
    m = meshgen.cylinder(8, 16, imperfection=50.0)
    t = m.meta["t"]
    a = capi.Assembler(m.X, m.conn, nonlinear=True)
    a.set_material(m.E, m.nu)
    a.set_thickness([t])
    a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    load = 0.3 * meshgen.classical_cylinder_load(m.E, m.nu, t, 1.0)
    u, its, rel = nonlinear.newton_preload(a, m.rhs, load=load, nsteps=4, rtol=1e-11)
    assert rel <= 1e-11 and len(its) == 4
    from test_gpu_solve import dense_buckling
    KT, G = a.create_mat(), a.create_mat()
    a.assemble_jacobian(KT, u, want_res=False)
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, u)
    sigma = 0.95 * dense_buckling(KT.to_dense_nodes(), G.to_dense_nodes(), m.bc_nodes,
                                  m.bc_mask)[0]
    lam_p, b_p, KT, G = nonlinear.preload_buckling(a, u, sigma, num_eigvals=2, eig_tol=1e-12,
                                                   block_size=2)
    assert abs(lam_p[1] - lam_p[0]) > 1e-3 * abs(lam_p[0])
    dX_p = nonlinear.preload_xpt_sens(a, u, lam_p[0], b_p.eigvecs[0], KT, G)
    b = capi.LinearBuckling(a, sigma, max_lanczos=120, num_eigvals=2, eig_tol=1e-12,
                            block_size=2)
    lam = b.solve_preloaded(u)
    assert np.max(np.abs(lam - lam_p) / np.abs(lam_p)) < 1e-10, (lam, lam_p)
    dX = b.eval_preload_xpt_sens(0)
    assert np.abs(dX - dX_p).max() <= 1e-6 * np.abs(dX_p).max()
    # the linear-path sensitivity entries refuse the preloaded state
    with pytest.raises(capi.A2dsError):
        b.eig_sens_thickness(0, 1)
