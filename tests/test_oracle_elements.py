"""The CPU oracle's shell element against fixtures written by the reference.

The fixtures (tests/golden/elements_*.npz) come from the reference's own
TACSShellElement instantiations (tests/golden/make_golden.py).  The oracle
restates the same algorithm in C, so K, the residual and the Jacobian agree
to a few ulps; G is a central difference in both (dh = 1e-4) and agrees to
the same level, and to ~5e-12 with the reference's complex-step G.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

TYPES = [("TACSQuad4Shell", 2, 0), ("TACSQuad4NonlinearShell", 2, 1),
         ("TACSQuad9Shell", 3, 0), ("TACSQuad9NonlinearShell", 3, 1)]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name,order,nl", TYPES)
def test_element_matrices_match_reference(name, order, nl):
    f = np.load(os.path.join(GOLDEN, f"elements_{name}.npz"))
    for s in range(f["X"].shape[0]):
        E, nu, t, alpha, temp, _ = f["params"][s]
        m = oracle.Material.iso(E, nu, t, alpha, temp)
        X, v = f["X"][s], f["vars"][s]
        K = oracle.element_matrix(order, nl, oracle.STIFFNESS, m, X, v)
        assert rel(K, f["K"][s]) < 1e-14
        R = oracle.element_residual(order, nl, m, X, v)
        assert rel(R, f["res"][s]) < 1e-13
        JR, J = oracle.element_jacobian(order, nl, m, X, v)
        assert rel(J, f["J"][s]) < 1e-14
        assert rel(JR, f["Jres"][s]) < 1e-13
        G = oracle.element_matrix(order, nl, oracle.GEOMETRIC, m, X, v)
        if nl and temp != 0.0:
            # The reference's nonlinear instantiations perturb their own
            # temperature member during getMatType(G) (nlElem == this), so
            # the backward step starts from the forward-perturbed value;
            # the oracle uses the unperturbed temperature for both steps.
            continue
        assert rel(G, f["G"][s]) < 1e-12
        if temp == 0.0:
            assert rel(G, f["G_cs"][s]) < 1e-11


@pytest.mark.parametrize("name,order,nl", TYPES)
def test_element_xpt_products_match_reference(name, order, nl):
    """Coordinate derivatives of psi^T K phi and psi^T G phi
    (TACSElement::addMatXptSensInnerProduct): the oracle's central
    differences (dh = 1e-7) against the reference's complex-step values.
    K: the reference's real-build formula, ~5e-9 from its complex step.
    G: a central difference (dh = 1e-4) inside the coordinate difference in
    both the oracle and the reference's real build (the two agree to
    ~1e-8), up to ~2e-5 from the complex step."""
    f = np.load(os.path.join(GOLDEN, f"elements_{name}.npz"))
    nn = order * order
    for s in range(f["X"].shape[0]):
        E, nu, t, alpha, temp, _ = f["params"][s]
        if temp != 0.0:
            continue
        m = oracle.Material.iso(E, nu, t, alpha, temp)
        args = (f["X"][s], f["vars"][s])
        psi, phi = f["xs_psi"][s], f["xs_phi"][s]
        KX = oracle.element_xpt_inner_product(order, nl, oracle.STIFFNESS, m, *args, psi, phi)
        assert rel(KX, f["KX_cs"][s].reshape(-1)) < 2e-8, (name, s)
        assert rel(KX, f["KX"][s].reshape(-1)) < 2e-8, (name, s)
        GX = oracle.element_xpt_inner_product(order, nl, oracle.GEOMETRIC, m, *args, psi, phi)
        assert rel(GX, f["GX"][s].reshape(-1)) < 2e-8, (name, s)
        assert rel(GX, f["GX_cs"][s].reshape(-1)) < 5e-5, (name, s)
    assert f["KX"].shape == (f["X"].shape[0], nn, 3)


@pytest.mark.parametrize("name,order,nl", TYPES)
def test_element_state_and_residual_products_match_reference(name, order, nl):
    """d(psi^T M phi)/d(vars) for K and G (TACSElement::
    getMatSVSensInnerProduct) and psi^T dR/dX (addAdjResXptProduct): the
    oracle's central differences (dh = 1e-7) against the reference's
    real-mode values (same formula) and its complex-step values."""
    f = np.load(os.path.join(GOLDEN, f"elements_{name}.npz"))
    for s in range(f["X"].shape[0]):
        E, nu, t, alpha, temp, _ = f["params"][s]
        if temp != 0.0:
            continue
        m = oracle.Material.iso(E, nu, t, alpha, temp)
        X, v = f["X"][s], f["vars"][s]
        psi, phi = f["xs_psi"][s], f["xs_phi"][s]
        KU = oracle.element_sv_inner_product(order, nl, oracle.STIFFNESS, m, X, v, psi, phi)
        if nl:
            assert rel(KU, f["KU"][s]) < 2e-8, (name, s)
            assert rel(KU, f["KU_cs"][s]) < 2e-8, (name, s)
        else:  # the linear tangent does not depend on the state
            assert not KU.any() and not f["KU"][s].any() and not f["KU_cs"][s].any()
        GU = oracle.element_sv_inner_product(order, nl, oracle.GEOMETRIC, m, X, v, psi, phi)
        assert rel(GU, f["GU"][s]) < 2e-8, (name, s)
        assert rel(GU, f["GU_cs"][s]) < 1e-6, (name, s)
        RX = oracle.element_adjres_xpt_product(order, nl, m, X, v, psi)
        assert rel(RX, f["RX"][s].reshape(-1)) < 2e-8, (name, s)
        assert rel(RX, f["RX_cs"][s].reshape(-1)) < 5e-8, (name, s)
