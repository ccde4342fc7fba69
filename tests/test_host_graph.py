"""Host-side integer artefacts against the reference's own arrays (bit-exact).

No GPU is needed: a2ds_mesh_plan builds the node-to-node pattern, the AMD
ordering, the BCSR pattern and the ILU(k) pattern on the host.  The expected
arrays come from the reference (tests/golden/cyl_*.npz, panel_*.npz):
computeLocalNodeToNodeCSR, amd_order_interface, the TACSSchurMat B pattern
and BCSRMat(comm, B, levFill, fill).
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from a2ds import capi

CASES = ["cyl_q4_4x8_lu", "cyl_q4_8x16_ilu1", "cyl_q9_2x4_lu", "panel_q9_4x8x1_lu"]


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    header = open(os.path.join(os.path.dirname(GOLDEN), "..", "include", "a2ds.h")).read()
    import re
    declared = set(re.findall(r"\b(a2ds_[a-z_0-9]+)\s*\(", header))
    assert declared, "no declarations found"
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared in include/a2ds.h but not exported"
    assert set(capi.EXPORTS) == declared


def _planned(f, order):
    a = capi.Assembler(f["X"], f["conn"])
    a.add_bcs(f["bc_nodes"], f["bc_mask"], f["bc_vals"])
    a.plan(order)
    return a


@pytest.mark.parametrize("case", CASES)
def test_node_csr_matches_reference(case):
    f = np.load(os.path.join(GOLDEN, case + ".npz"))
    a = capi.Assembler(f["X"], f["conn"])
    rowp, cols = a.node_csr(nodiag=False)
    assert np.array_equal(rowp, f["csr_rowp"])
    assert np.array_equal(cols, f["csr_cols"])


@pytest.mark.parametrize("case", CASES)
def test_amd_ordering_and_patterns_match_reference(case):
    f = np.load(os.path.join(GOLDEN, case + ".npz"))
    a = _planned(f, capi.A2DS_TACS_AMD_ORDER)
    assert np.array_equal(a.get_ordering(), f["amd_perm"])
    rowp, cols = a.get_pattern()
    assert np.array_equal(rowp, f["bcsr_rowp"])
    assert np.array_equal(cols, f["bcsr_cols"])
    frowp, fcols = a.ilu_pattern(int(f["lev"]))
    assert np.array_equal(frowp, f["ilu_rowp"])
    assert np.array_equal(fcols, f["ilu_cols"])


def test_natural_ordering_is_identity():
    f = np.load(os.path.join(GOLDEN, CASES[0] + ".npz"))
    a = _planned(f, capi.A2DS_NATURAL_ORDER)
    assert np.array_equal(a.get_ordering(), np.arange(f["X"].shape[0]))


def test_bad_inputs_are_rejected():
    X = np.zeros((4, 3))
    with pytest.raises(capi.A2dsError):
        capi.Assembler(X, np.array([[0, 1, 2, 7]]))      # node out of range
    with pytest.raises(capi.A2dsError):
        capi.Assembler(X, np.array([[0, 1, 2]]))         # 3-node element


ORDER_CASES = ["cyl_q4_4x8", "cyl_q4_8x16", "cyl_q9_2x4", "cyl_q4_16x32"]


@pytest.mark.parametrize("case", ORDER_CASES)
@pytest.mark.parametrize("order,key", [(capi.A2DS_RCM_ORDER, "rcm_new_vars"),
                                       (capi.A2DS_MULTICOLOR_ORDER, "mc_new_vars")])
def test_rcm_and_multicolor_orderings_match_reference(case, order, key):
    """createSchurMat(RCM_ORDER / MULTICOLOR_ORDER) on one process: the
    permutation from TacsComputeRCMOrder (root 0, one pass) and
    TacsComputeSerialMultiColor on the node graph with its diagonal
    (tests/golden/orderings.npz, written by the reference's own routines)."""
    f = np.load(os.path.join(GOLDEN, "orderings.npz"))
    a = capi.Assembler(f[f"{case}__X"], f[f"{case}__conn"])
    a.plan(order)
    new_vars = f[f"{case}__{key}"]
    expect = np.empty_like(new_vars)
    expect[new_vars] = np.arange(new_vars.size, dtype=new_vars.dtype)
    assert np.array_equal(a.get_ordering(), expect)


def test_amd_order_type_equals_tacs_amd_and_nd_is_refused():
    f = np.load(os.path.join(GOLDEN, "cyl_q4_8x16_ilu1.npz"))
    a = _planned(f, capi.A2DS_AMD_ORDER)
    assert np.array_equal(a.get_ordering(), f["amd_perm"])
    b = capi.Assembler(f["X"], f["conn"])
    with pytest.raises(capi.A2dsError, match="METIS"):
        b.plan(capi.A2DS_ND_ORDER)


@pytest.mark.parametrize("order", [capi.A2DS_TACS_AMD_ORDER, capi.A2DS_RCM_ORDER,
                                   capi.A2DS_NATURAL_ORDER, capi.A2DS_MULTICOLOR_ORDER])
def test_complete_fill_paths_agree(order):
    """Complete fill of a symmetric pattern takes the elimination-tree path;
    levFill = n - 2 (still complete: no fill level exceeds the number of
    intermediate rows) takes the row-by-row level-of-fill path of
    computeILUk.  The two patterns are identical."""
    from a2ds import mesh as meshgen
    for m in (meshgen.cylinder(16, 32), meshgen.cylinder(4, 8, order=3),
              meshgen.stiffened_panel(2, 8, 1)):
        a = capi.Assembler(m.X, m.conn)
        a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
        a.plan(order)
        r1, c1 = a.ilu_pattern(1000000)
        r2, c2 = a.ilu_pattern(m.num_nodes - 2)
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
