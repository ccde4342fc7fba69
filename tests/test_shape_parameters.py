"""The cylinder's radial shape parameters (64 seeded parameters on an 8 x 8
grid of axial and circumferential wave numbers) that the coordinate
sensitivities chain through."""
import numpy as np

from a2ds import mesh as meshgen


def test_shape_parameterisation():
    """The 64 radial shape parameters: modes vanish on both end rings, the
    moved coordinates are linear in s, and the chain rule for dlambda/ds is
    the contraction with the modes."""
    m = meshgen.cylinder(8, 16)
    modes = meshgen.radial_shape_modes(m)
    assert modes.shape == (64, m.num_nodes, 3)
    ends = (np.abs(m.X[:, 0]) < 1e-12) | (np.abs(m.X[:, 0] - 2.0) < 1e-12)
    assert np.abs(modes[:, ends]).max() < 1e-12
    s = meshgen.seeded_shape_parameters()
    X1 = meshgen.shaped_coordinates(m, s, modes)
    X2 = meshgen.shaped_coordinates(m, 2 * s, modes)
    assert np.allclose(X2 - m.X, 2 * (X1 - m.X), rtol=0, atol=1e-15)
    assert np.array_equal(meshgen.shaped_coordinates(m, np.zeros(64), modes), m.X)
    # radial: the x coordinate does not move
    assert np.abs(X1[:, 0] - m.X[:, 0]).max() == 0.0
