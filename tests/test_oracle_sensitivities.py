"""The eigenvalue coordinate-sensitivity formula (the body of the reference's
commented-out TACSLinearBuckling::evalEigenXptSens, restated densely in
oracle/sens.py from the oracle's element routines) against central
differences of whole dense solves on moved meshes, for linear buckling and
for buckling about a nonlinear preloaded state (4x8 Quad4 cylinders with a
large imperfection, so the lowest load is simple), along axisymmetric
radial shape modes; rigid motions leave the load unchanged.  The thickness
derivative (the documented evalEigenDVSens formula) the same way."""
import numpy as np
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
