"""The eigenvalue coordinate-sensitivity formula (the body of the reference's
commented-out TACSLinearBuckling::evalEigenXptSens, restated densely in
oracle/sens.py from the oracle's element routines) against central
differences of whole dense solves on moved meshes, for linear buckling and
for buckling about a nonlinear preloaded state (4x8 Quad4 cylinders with a
large imperfection, so the lowest load is simple), along axisymmetric
radial shape modes; rigid motions leave the load unchanged.  The thickness
derivative (the documented evalEigenDVSens formula) the same way."""
import numpy as np

import oracle
import pytest

from a2ds import mesh as meshgen
from oracle.sens import DenseShell


@pytest.mark.parametrize("nonlinear", [False, True])
def test_dense_xpt_sensitivity_vs_finite_difference(nonlinear):
    m = meshgen.cylinder(4, 8, imperfection=50.0)
    ds = DenseShell(m, nonlinear)
    load = 0.3 * meshgen.classical_cylinder_load(m.E, m.nu, m.meta["t"], 1.0) if nonlinear else None

    def solve(X):
        u = ds.state(X, load)
        return (u,) + ds.buckling(X, u)

    u, lam, phi, K, G = solve(m.X)
    assert abs(lam[1]) > 1.02 * abs(lam[0])  # a simple lowest load
    dX = ds.xpt_sens(m.X, u, lam[0], phi[:, 0], K, G)
    # the element central differences (dh = 1e-7) carry ~1e-6 rounding noise
    # relative to sum |dX|: the invariances hold to that level
    scale = np.abs(dX).sum()
    assert np.all(np.abs(dX.sum(axis=0)) <= 1e-5 * scale)
    spin = np.stack([np.zeros(m.num_nodes), -m.X[:, 2], m.X[:, 1]], axis=1)
    assert abs(np.sum(dX * spin)) <= 1e-5 * scale
    modes = meshgen.radial_shape_modes(m)
    eps = 1e-5
    for p in (0, 16):
        d = float(np.sum(dX * modes[p]))
        fd = (solve(m.X + eps * modes[p])[1][0] - solve(m.X - eps * modes[p])[1][0]) / (2 * eps)
        assert abs(d - fd) <= 1e-4 * abs(fd), (p, d, fd)


def test_dense_thickness_sensitivity_vs_finite_difference():
    """The documented evalEigenDVSens formula (with the load-path adjoint)
    restated densely, against central differences of whole solves in the
    shell thickness."""
    m = meshgen.cylinder(4, 8, imperfection=50.0)
    t = float(m.thickness[0])
    ds = DenseShell(m)
    u = ds.state(m.X)
    lam, phi, K, G = ds.buckling(m.X, u)
    d = ds.thickness_sens(m.X, u, lam[0], phi[:, 0], K, G)

    def load(tt):  # same coordinates and loads, thickness tt
        import dataclasses
        mm = dataclasses.replace(m, thickness=np.full_like(m.thickness, tt))
        dd = DenseShell(mm)
        uu = dd.state(mm.X)
        return dd.buckling(mm.X, uu)[0][0]
    h = 1e-6 * t
    fd = (load(t + h) - load(t - h)) / (2 * h)
    assert abs(d - fd) <= 1e-5 * abs(fd), (d, fd)


def test_dense_group_thickness_sensitivities_sum_to_the_uniform_derivative():
    """Per-group thickness derivatives of the stiffened panel's lowest load
    (oracle/sens.py thickness_sens_groups, 64 groups in use) at a uniform
    thickness sum to the derivative for a uniform change of all of them (the
    one-thickness formula of DenseShell.thickness_sens, itself checked
    against whole-solve differences above).  (Whole-solve differences of the
    dense panel solves carry ~1e-4 noise: the dense generalized eigensolve's
    error grows with cond(K) ~ 1e10, so they cannot pin 1e-6.)"""
    import dataclasses
    from oracle.sens import DenseShell, dense_buckling_groups, thickness_sens_groups
    m = meshgen.stiffened_panel(4, 8, 1)
    m = dataclasses.replace(m, thickness=np.full_like(m.thickness, m.thickness[0]))
    u, lam, phi, K, G = dense_buckling_groups(m)
    d = thickness_sens_groups(m, u, lam[0], phi[:, 0], K, G)
    assert np.count_nonzero(d) == np.unique(m.dv_group).size == 64
    ds = DenseShell(m)
    ref = ds.thickness_sens(m.X, u, lam[0], phi[:, 0], K, G)
    assert abs(d.sum() - ref) <= 1e-10 * abs(ref), (d.sum(), ref)


def test_element_matrices_are_t_plus_t_cubed():
    """The exact thickness derivative of thickness_sens_groups rests on
    M_e(t) = t M1 + t^3 M3 (no thickness offset): checked at a third
    thickness for K and G of a Quad4 and a Quad9 element."""
    from oracle.sens import _dt_element
    for order in (2, 3):
        m = meshgen.cylinder(1, 4, order=order)
        c = m.conn[0]
        v = 1e-3 * np.random.default_rng(0).standard_normal(6 * order * order)
        for kind, vv in ((oracle.STIFFNESS, np.zeros_like(v)), (oracle.GEOMETRIC, v)):
            M = lambda t: oracle.element_matrix(order, 0, kind, oracle.Material.iso(m.E, m.nu, t),
                                                m.X[c], vv)
            M3 = (M(2.0) - 2.0 * M(1.0)) / 6.0
            M1 = M(1.0) - M3
            t = 3.7e-3
            assert np.abs(M(t) - (t * M1 + t ** 3 * M3)).max() <= 1e-10 * np.abs(M(t)).max()
            h = 1e-3 * t
            fd = (M(t + h) - M(t - h)) / (2 * h)
            dt = _dt_element(order, kind, m.E, m.nu, t, m.X[c], vv)
            assert np.abs(dt - fd).max() <= 1e-6 * np.abs(fd).max()
