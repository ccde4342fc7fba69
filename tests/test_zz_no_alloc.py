"""a2ds_bcsr_mult_rows_noalloc against a2ds_bcsr_mult_rows.

The no-allocation entry point stages x and y through a fixed device array
instead of per-call buffers; its product must equal the allocating entry
point's on the same matrix.  Two calls in a row with different vectors check
that nothing from the first call leaks into the second (the scratch array is
shared and never cleared).  Tolerance: normwise relative 1e-13 (both run the
same FP64 kernel, so equality is expected).  This file is collected last so
that it also runs after every other GPU test in the same process.
"""
import numpy as np
import pytest

from a2ds import capi
from a2ds import mesh as meshgen

MAX_ROWS = 65536


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def cylinder_assembler(nx, ny):
    m = meshgen.cylinder(nx, ny, order=2)
    a = capi.Assembler(m.X, m.conn)
    a.set_material(m.E, m.nu)
    a.set_thickness(m.thickness[:1])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    return a


@pytest.mark.gpu
def test_noalloc_mult_matches_allocating_entry_point():
    a = cylinder_assembler(24, 48)
    K = a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K)
    rowp, cols, vals = K.get_arrays()
    nn = rowp.size - 1
    rng = np.random.default_rng(11)
    prev = None
    for call in range(2):
        x = rng.standard_normal((nn, 6))
        y_ref = K.mult_rows(x)
        y = K.mult_rows(x, noalloc=True)
        assert rel(y, y_ref) < 1e-13
        # independent host check of the product in row ordering
        y_np = np.zeros_like(x)
        for r in range(nn):
            for k in range(rowp[r], rowp[r + 1]):
                y_np[r] += vals[k] @ x[cols[k]]
        assert rel(y, y_np) < 1e-13
        if prev is not None:
            assert not np.array_equal(y, prev)
        prev = y


@pytest.mark.gpu
def test_noalloc_smaller_matrix_after_larger():
    """A 4x8 cylinder right after a 24x48 one: the shared array's tail still
    holds the larger call's values, and the smaller product must not see
    them."""
    big = cylinder_assembler(24, 48)
    Kb = big.create_mat()
    big.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, Kb)
    rng = np.random.default_rng(5)
    xb = rng.standard_normal((big.num_nodes, 6))
    assert rel(Kb.mult_rows(xb, noalloc=True), Kb.mult_rows(xb)) < 1e-13
    small = cylinder_assembler(4, 8)
    Ks = small.create_mat()
    small.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, Ks)
    rowp, cols, vals = Ks.get_arrays()
    nn = rowp.size - 1
    xs = rng.standard_normal((nn, 6))
    y = Ks.mult_rows(xs, noalloc=True)
    assert rel(y, Ks.mult_rows(xs)) < 1e-13
    y_np = np.zeros_like(xs)
    for r in range(nn):
        for k in range(rowp[r], rowp[r + 1]):
            y_np[r] += vals[k] @ xs[cols[k]]
    assert rel(y, y_np) < 1e-13


@pytest.mark.gpu
def test_noalloc_rejects_oversize_matrix():
    a = cylinder_assembler(256, 256)
    assert a.num_nodes > MAX_ROWS
    K = a.create_mat()
    x = np.zeros((a.num_nodes, 6))
    with pytest.raises(capi.A2dsError, match="at most 65536 block rows"):
        K.mult_rows(x, noalloc=True)
