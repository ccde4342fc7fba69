"""The stiffened-panel workload: a flat Quad9 skin with eight blade webs
joined along their roots (T-junctions), 20 axial segments x 20 lanes of
thickness design groups drawn from U[2, 20] mm, compressed by 1 kN/m at
x = L (a2ds.mesh.stiffened_panel).  The reference assembled and solved the
4 x 8 x 1 instance (tests/golden/panel_q9_4x8x1_lu.npz; one constitutive
object per distinct thickness):

* CPU: the generator's sizes and loads at the full 1360 x 408 x 41 size
  (about 1.0 M Quad9 elements, 24 M DOF) and at the fixture's size.
* GPU: K and G against the reference's (1e-12 and its FD noise), the load
  path against its path, and the loads of smallest magnitude (this panel
  has negative ones too: buckling under the reversed load) against the
  dense FP64 eigenvalues of the reference's own K and G (1e-8), in FP64 and
  double-float factors; d(lambda)/d(t_g) for all 400 groups against central
  differences (step 1e-6 t) on the most influential and on seeded groups.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from a2ds import capi
from a2ds import mesh as meshgen

CASE = "panel_q9_4x8x1_lu"


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_generator_sizes_and_loads():
    m = meshgen.stiffened_panel(4, 8, 1)
    f = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    assert np.array_equal(m.X, f["X"]) and np.array_equal(m.conn, f["conn"])
    assert np.array_equal(m.thickness, f["thickness"])
    assert np.isclose(m.rhs[:, 0].sum(), -1e3 * (0.6 + 8 * 0.06))
    assert m.meta["tvals"].size == 400 and m.dv_group.max() < 400
    # the web roots are skin nodes: every web element has three skin nodes
    web = m.conn[4 * 8:]
    assert np.all((m.X[web][:, :, 2] == 0.0).sum(axis=1) == 3)
    with pytest.raises(ValueError):
        meshgen.stiffened_panel(4, 6, 1)  # no skin node lines at the roots


def test_generator_full_size():
    m = meshgen.stiffened_panel(1360, 408, 41)
    assert (m.num_elements, m.num_nodes) == (1360 * 408 + 8 * 1360 * 41,
                                             2721 * 817 + 8 * 2721 * 82)
    assert 6 * m.num_nodes > 24_000_000
    assert np.unique(m.dv_group).size == 400


def assembler(f):
    ne = f["conn"].shape[0]
    a = capi.Assembler(f["X"], f["conn"])
    a.set_material(float(f["E"]), float(f["nu"]))
    a.set_thickness(f["thickness"], np.arange(ne, dtype=np.int32))
    a.add_bcs(f["bc_nodes"], f["bc_mask"], f["bc_vals"])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    return a


@pytest.mark.gpu
def test_panel_assembly_vs_reference():
    f = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    a = assembler(f)
    K = a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K)
    rowp, cols, vals = K.get_arrays()
    assert np.array_equal(rowp, f["bcsr_rowp"]) and np.array_equal(cols, f["bcsr_cols"])
    assert rel(vals, f["K_after"]) < 1e-12
    G = a.create_mat()
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, f["path"])
    assert rel(G.get_arrays()[2], f["G"]) < 5e-11


def reference_dense_loads(f):
    """Eigenvalues of K x + lam G x = 0 (free DOFs, all signs, by magnitude)
    from the reference's assembled K and G (row ordering of its AMD
    permutation)."""
    import scipy.linalg as sla
    rowp, cols = f["bcsr_rowp"], f["bcsr_cols"]
    n = rowp.size - 1

    def dense(vals):
        A = np.zeros((6 * n, 6 * n))
        for i in range(n):
            for jp in range(rowp[i], rowp[i + 1]):
                A[6 * i:6 * i + 6, 6 * cols[jp]:6 * cols[jp] + 6] = vals[jp]
        return A
    inv = np.empty(n, np.int64)
    inv[f["amd_perm"]] = np.arange(n)
    free = np.ones(6 * n, bool)
    for node, mask in zip(f["bc_nodes"], f["bc_mask"]):
        for k in range(6):
            if mask >> k & 1:
                free[6 * inv[node] + k] = False
    K, G = dense(f["K_after"]), dense(f["G"])
    Kf, Gf = K[np.ix_(free, free)], G[np.ix_(free, free)]
    mu = sla.eigh(-0.5 * (Gf + Gf.T), 0.5 * (Kf + Kf.T), eigvals_only=True)
    lam = 1.0 / mu[mu != 0]
    return lam[np.argsort(np.abs(lam))]


def test_reference_dense_loads_include_the_fixture_list():
    """The fixture's eigvals_dense lists the positive loads only."""
    f = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    lam = reference_dense_loads(f)[:10]
    pos = np.sort(lam[lam > 0])
    assert np.allclose(pos, f["eigvals_dense"][:pos.size], rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 48])
def test_panel_buckling_matches_reference(precision):
    f = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    a = assembler(f)
    nev = 5
    b = capi.LinearBuckling(a, float(f["sigma"]), max_lanczos=120, num_eigvals=nev,
                            eig_tol=1e-12, lev_fill=1000000, precision=precision, block_size=4)
    lam = b.solve(f["rhs"])
    assert np.all(b.errors < 1e-8), b.errors
    assert rel(b.path, f["path"]) < 1e-8
    ref = reference_dense_loads(f)[:nev]
    assert np.max(np.abs(lam - ref) / np.abs(ref)) < 1e-8, (lam, ref)


@pytest.mark.gpu
def test_panel_thickness_sensitivities_vs_finite_difference():
    m = meshgen.stiffened_panel(4, 8, 1)
    f = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    tv = m.meta["tvals"]

    def solve(t):
        a = capi.Assembler(m.X, m.conn)
        a.set_material(m.E, m.nu)
        a.set_thickness(t, m.dv_group)
        a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
        a.initialize(capi.A2DS_TACS_AMD_ORDER)
        b = capi.LinearBuckling(a, float(f["sigma"]), max_lanczos=120, num_eigvals=2,
                                eig_tol=1e-13, precision=48, block_size=4)
        return b, b.solve(m.rhs)

    b, lam = solve(tv)
    dl = b.eig_sens_thickness(0, tv.size)
    used = np.unique(m.dv_group)
    assert np.all(dl[np.setdiff1d(np.arange(tv.size), used)] == 0.0)
    # the two most influential groups and two seeded ones; the absolute term
    # is the eigenvalue noise (~1e-12 relative) over the step
    rng = np.random.default_rng(7)
    top = used[np.argsort(-np.abs(dl[used]))[:2]]
    for g in list(top) + list(rng.choice(np.setdiff1d(used, top), 2, replace=False)):
        h = 1e-6 * tv[g]
        tp, tm = tv.copy(), tv.copy()
        tp[g] += h
        tm[g] -= h
        fd = (solve(tp)[1][0] - solve(tm)[1][0]) / (2 * h)
        assert abs(dl[g] - fd) <= 1e-4 * abs(fd) + 2e-6 * abs(lam[0]) / tv[g], (g, dl[g], fd)

