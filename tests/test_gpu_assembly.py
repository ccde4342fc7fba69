"""GB300 element assembly against the reference and the CPU oracle.

Element level: a one-element mesh reproduces each fixture element of
tests/golden/elements_*.npz (written by the reference's own
TACSShellElement).  Mesh level: the seeded cylinders of tests/golden/cyl_*.npz
(assembled K at the zero state and G along the reference's load path, with
the row-only Dirichlet treatment).  Tolerances are normwise relative
(max |A - B| / max |B|):

  K, J, residual   1e-12
  G vs the reference's complex-step G            1e-12
  G vs the reference's finite-difference G       5e-11 (its FD noise is ~5e-12)
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from a2ds import capi

TYPES = [("TACSQuad4Shell", 2, 0), ("TACSQuad4NonlinearShell", 2, 1),
         ("TACSQuad9Shell", 3, 0), ("TACSQuad9NonlinearShell", 3, 1)]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def fd_geometric(order, E, nu, t, alpha, temp, X, v, dh):
    """The reference's central difference of the nonlinear tangent
    (TACSShellElement.h:700-767) through the oracle, with step dh."""
    norm = np.sqrt((v ** 2).sum() + temp ** 2)
    a = 0.5 * norm / dh
    mp = oracle.Material.iso(E, nu, t, alpha, temp + dh * temp / norm)
    mm = oracle.Material.iso(E, nu, t, alpha, temp - dh * temp / norm)
    _, J1 = oracle.element_jacobian(order, 1, mp, X, dh * v / norm, a)
    _, J2 = oracle.element_jacobian(order, 1, mm, X, -dh * v / norm, -a)
    return J1 + J2


def one_element(X, order, nl, E, nu, t, alpha, temp):
    nn = order * order
    a = capi.Assembler(X.reshape(nn, 3), np.arange(nn, dtype=np.int32)[None, :], nonlinear=nl)
    a.set_material(E, nu, alpha, temp)
    a.set_thickness([t])
    a.initialize(capi.A2DS_NATURAL_ORDER)
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("name,order,nl", TYPES)
def test_element_xpt_products_vs_reference(name, order, nl):
    """d(psi^T K phi)/dX and d(psi^T G phi)/dX (TACSElement::
    addMatXptSensInnerProduct) on one-element meshes: GPU central
    differences (dh = 1e-7, the reference's real-mode step) against the
    reference's complex-step values (exact for K; for G the derivative of its
    central-difference G, which is exact up to rounding here) and its
    real-mode values (same formula for K)."""
    f = np.load(os.path.join(GOLDEN, f"elements_{name}.npz"))
    nn = order * order
    for s in range(f["X"].shape[0]):
        E, nu, t, alpha, temp, _ = f["params"][s]
        if temp != 0.0:
            continue
        a = one_element(f["X"][s], order, nl, E, nu, t, alpha, temp)
        v = f["vars"][s].reshape(nn, 6)
        psi, phi = f["xs_psi"][s].reshape(nn, 6), f["xs_phi"][s].reshape(nn, 6)
        KX = a.add_mat_xpt_sens_inner_product(1.0, capi.A2DS_STIFFNESS_MATRIX, psi, phi, vars_=v)
        assert rel(KX, f["KX_cs"][s]) < 2e-8, (name, s, "K")
        assert rel(KX, f["KX"][s]) < 2e-8, (name, s, "K vs real-mode")
        GX = a.add_mat_xpt_sens_inner_product(1.0, capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, psi, phi,
                                              vars_=v)
        assert rel(GX, f["GX_cs"][s]) < 2e-8, (name, s, "G")
        # state derivatives (getMatSVSensInnerProduct) and the
        # adjoint-residual coordinate product (addAdjResXptProduct)
        KU = a.eval_mat_sv_sens_inner_product(capi.A2DS_STIFFNESS_MATRIX, psi, phi, v)
        if nl:
            assert rel(KU, f["KU_cs"][s].reshape(nn, 6)) < 2e-8, (name, s, "K state")
        else:  # the linear tangent does not depend on the state
            scale = np.abs(f["K"][s]).max() * np.abs(psi).max() * np.abs(phi).max()
            assert np.abs(KU).max() <= 1e-6 * scale, (name, s, "linear K state")
        GU = a.eval_mat_sv_sens_inner_product(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, psi, phi, v)
        assert rel(GU, f["GU_cs"][s].reshape(nn, 6)) < 2e-8, (name, s, "G state")
        RX = a.add_adjoint_res_xpt_sens_products(1.0, psi, vars_=v)
        assert rel(RX, f["RX_cs"][s]) < 5e-8, (name, s, "residual")
        assert rel(RX, f["RX"][s]) < 2e-8, (name, s, "residual vs real-mode")
        # scale and accumulation (atomic order of multi-warp elements: the
        # stepped contractions cancel to ~1e-10 of the derivative)
        acc = a.add_mat_xpt_sens_inner_product(-2.0, capi.A2DS_STIFFNESS_MATRIX, psi, phi,
                                               dfdX=KX.copy(), vars_=v)
        assert rel(acc, -KX) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("name,order,nl", TYPES)
def test_element_matrices_vs_reference(name, order, nl):
    f = np.load(os.path.join(GOLDEN, f"elements_{name}.npz"))
    nn = order * order
    for s in range(f["X"].shape[0]):
        E, nu, t, alpha, temp, _ = f["params"][s]
        a = one_element(f["X"][s], order, nl, E, nu, t, alpha, temp)
        v = f["vars"][s].reshape(nn, 6)
        K = a.create_mat()
        a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K, v)
        assert rel(K.to_dense_nodes(), f["K"][s]) < 1e-12, (name, s, "K")
        G = a.create_mat()
        a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, v)
        Gd = G.to_dense_nodes()
        if temp == 0.0:
            assert rel(Gd, f["G_cs"][s]) < 1e-12, (name, s, "G vs complex step")
            assert rel(Gd, f["G"][s]) < 5e-11, (name, s, "G vs finite difference")
        elif not nl:
            # Thermal: the real-mode reference perturbs the temperature too
            # (its complex-step build does not), and its dh = 1e-4 central
            # difference carries ~1e-9 rounding noise on top of the large
            # thermal prestress.  The oracle's central difference at
            # dh = 1e-2 (exact in exact arithmetic, ~1e-11 noise) is the
            # tight check; the reference's FD G the loose one.
            assert rel(Gd, fd_geometric(order, E, nu, t, alpha, temp, f["X"][s],
                                        f["vars"][s], 1e-2)) < 1e-10, (name, s, "thermal G")
            assert rel(Gd, f["G"][s]) < 5e-9, (name, s, "thermal G vs reference FD")
        R = a.assemble_res(v)
        assert rel(R.ravel(), f["res"][s]) < 1e-12, (name, s, "residual")
        J = a.create_mat()
        JR = a.assemble_jacobian(J, v)
        assert rel(J.to_dense_nodes(), f["J"][s]) < 1e-12, (name, s, "J")
        assert rel(JR.ravel(), f["Jres"][s]) < 1e-12, (name, s, "J residual")


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cyl_q4_4x8_lu", "cyl_q4_8x16_ilu1", "cyl_q9_2x4_lu"])
@pytest.mark.parametrize("scatter", [capi.A2DS_SCATTER_ATOMIC, capi.A2DS_SCATTER_COLORED])
def test_cylinder_assembly_vs_reference(case, scatter):
    f = np.load(os.path.join(GOLDEN, case + ".npz"))
    a = capi.Assembler(f["X"], f["conn"])
    a.set_material(float(f["E"]), float(f["nu"]))
    a.set_thickness(f["thickness"][:1])
    a.add_bcs(f["bc_nodes"], f["bc_mask"], f["bc_vals"])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    K = a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K, None, scatter)
    rowp, cols, vals = K.get_arrays()
    assert np.array_equal(rowp, f["bcsr_rowp"]) and np.array_equal(cols, f["bcsr_cols"])
    assert rel(vals, f["K_after"]) < 1e-12
    G = a.create_mat()
    # G_cs was formed by the complex-step build at its own load path
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, f["path_cs"], scatter)
    _, _, gv = G.get_arrays()
    assert rel(gv, f["G_cs"]) < 1e-12
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, f["path"], scatter)
    _, _, gv = G.get_arrays()
    assert rel(gv, f["G"]) < 5e-11
    # BCSRMat::copyValues / axpy / applyBCs (the shifted operator of
    # TACSLinearBuckling::solve: aux <- K, aux += sigma G, aux.applyBCs)
    # against the same operations on the reference's arrays and on this
    # library's own K and G
    A = a.create_mat()
    A.copy_values(K)
    assert np.array_equal(A.get_arrays()[2], vals)
    sigma = 0.37
    A.axpy(sigma, G)
    av = A.get_arrays()[2]
    assert rel(av, f["K_after"] + sigma * f["G"]) < 5e-11
    # one rounding per entry (FMA or multiply-add) of |K| + |sigma G|
    scale = np.abs(vals) + np.abs(sigma * gv)
    close = np.abs(av - (vals + sigma * gv)) <= 4e-16 * scale
    assert np.all(close)
    A.apply_bcs()
    av = A.get_arrays()[2]
    # applyBCs only rewrites constrained rows, into K's (identity) rows
    close = np.abs(av - (vals + sigma * gv)) <= 4e-16 * scale
    assert np.all(close | (av == vals))
    # y = K x through the GPU SpMV against the reference's BCSRMat::mult
    xr = np.sin(1.0 + np.arange(6 * (rowp.size - 1)))
    y = np.zeros_like(xr)
    capi._check(a.lib.a2ds_bcsr_mult_rows(K.h, capi._d(xr), capi._d(y)))
    assert rel(y, f["K_mult_y"]) < 1e-13


@pytest.mark.gpu
def test_colored_scatter_is_bitwise_reproducible():
    f = np.load(os.path.join(GOLDEN, "cyl_q4_8x16_ilu1.npz"))
    a = capi.Assembler(f["X"], f["conn"])
    a.set_material(float(f["E"]), float(f["nu"]))
    a.set_thickness(f["thickness"][:1])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    out = []
    for _ in range(2):
        G = a.create_mat()
        a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, f["path"],
                            capi.A2DS_SCATTER_COLORED)
        out.append(G.get_arrays()[2])
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
def test_mesh_assembly_matches_oracle_elementwise():
    """Random seeded geometry/state on a small cylinder: the assembled GPU
    matrix equals the sum of oracle element matrices."""
    from a2ds import mesh as meshgen
    m = meshgen.cylinder(3, 6, order=2)
    rng = np.random.default_rng(7)
    u = 1e-3 * rng.standard_normal((m.num_nodes, 6))
    a = capi.Assembler(m.X, m.conn, nonlinear=True)
    a.set_material(m.E, m.nu)
    a.set_thickness([2e-3])
    a.initialize(capi.A2DS_NATURAL_ORDER)
    K = a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K, u)
    mat = oracle.Material.iso(m.E, m.nu, 2e-3)
    ref = np.zeros((6 * m.num_nodes, 6 * m.num_nodes))
    for e in range(m.num_elements):
        nodes = m.conn[e]
        Ke = oracle.element_matrix(2, 1, oracle.STIFFNESS, mat, m.X[nodes], u[nodes].ravel())
        idx = (6 * nodes[:, None] + np.arange(6)[None, :]).ravel()
        ref[np.ix_(idx, idx)] += Ke
    assert rel(K.to_dense_nodes(), ref) < 1e-12


@pytest.mark.gpu
def test_bcsr_time_mult():
    """The measurement entries behind bench.py's SpMV figures (FP64 product
    and the double-float product of the GMRES-IR inner loop): positive device
    times for 1 and 4 vectors, argument checks."""
    f = np.load(os.path.join(GOLDEN, "cyl_q4_8x16_ilu1.npz"))
    a = capi.Assembler(f["X"], f["conn"])
    a.set_material(float(f["E"]), float(f["nu"]))
    a.set_thickness(f["thickness"][:1])
    a.add_bcs(f["bc_nodes"], f["bc_mask"], f["bc_vals"])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    K = a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K)
    assert K.sizes() == (f["bcsr_rowp"].size - 1, f["bcsr_cols"].size)
    for p in (1, 4):
        ms = K.time_mult(p, 5)
        assert np.isfinite(ms) and ms > 0.0
        ms = K.time_mult_df(p, 5)
        assert np.isfinite(ms) and ms > 0.0
    with pytest.raises(capi.A2dsError):
        K.time_mult(3, 5)
    with pytest.raises(capi.A2dsError):
        K.time_mult(1, 0)
    with pytest.raises(capi.A2dsError):
        K.time_mult_df(3, 5)
