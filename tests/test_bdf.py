"""BDF mesh input (TACSMeshLoader::scanBDFFile, src/io/TACSMeshLoader.cpp:
569-1098) against the reference loader's own output on synthetic decks
(tests/golden/bdf_*.bdf, bdf.npz; written by tests/golden/bdf_cases.py and
parsed by the reference through oracle/ref/golden_gen.cpp).

* CPU: connectivity, components, nodes, SPC entries and names bit-exact;
  the failures the reference aborts on are errors.
* GPU: the cylinder deck (displacement control through nonzero SPC values)
  through the loader and the GB300 buckling solve matches the reference's
  TACSLinearBuckling eigenvalues on the same parsed mesh to 1e-8.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from a2ds import capi

DECKS = ["bdf_mixed", "bdf_plain", "bdf_cyl_q4_8x16"]


def golden(name):
    d = np.load(os.path.join(GOLDEN, "bdf.npz"))
    return {k[len(name) + 2:]: d[k] for k in d.files if k.startswith(name + "__")}


@pytest.mark.parametrize("name", DECKS)
def test_loader_matches_reference(name):
    g = golden(name)
    fail, nn, ne, nbcs, ncomp = g["sizes"]
    assert fail == 0
    ml = capi.MeshLoader()
    ml.scan_bdf_file(os.path.join(GOLDEN, name + ".bdf"))
    assert (ml.get_num_nodes(), ml.get_num_elements(), ml.get_num_components()) == (nn, ne, ncomp)
    ptr, conn, comp, X = ml.get_connectivity()
    assert np.array_equal(ptr, g["elem_node_ptr"])
    assert np.array_equal(conn, g["elem_node_conn"])
    assert np.array_equal(comp, g["elem_component"])
    assert np.array_equal(X, g["Xpts"])  # same digits, same conversion: exact
    nodes, var, bptr, vals = ml.get_bcs()
    assert np.array_equal(nodes, g["bc_nodes"])
    assert np.array_equal(bptr, g["bc_ptr"])
    assert np.array_equal(var, g["bc_vars"])
    assert np.array_equal(vals, g["bc_vals"])
    names = [bytes(r).rstrip(b"\0").decode() for r in g["names"]]
    assert [ml.get_element_descript(c) for c in range(ncomp)] == names[:ncomp]
    assert [ml.get_component_descript(c) for c in range(ncomp)] == names[ncomp:]


def test_loader_errors(tmp_path):
    ml = capi.MeshLoader()
    with pytest.raises(capi.A2dsError):
        ml.scan_bdf_file(str(tmp_path / "missing.bdf"))
    bad = {
        # an empty line inside the bulk data (the reference aborts)
        "empty": "BEGIN BULK\nGRID           1       0     0.0     0.0     0.0\n\nENDDATA\n",
        # an element on a node that no GRID defines
        "undefined": ("BEGIN BULK\nGRID           1       0     0.0     0.0     0.0\n"
                      "CTRIA3         1       1       1       2       3\nENDDATA\n"),
        # a CQUAD4 with three nodes (below the card's node count)
        "short": ("BEGIN BULK\nGRID           1       0     0.0     0.0     0.0\n"
                  "CQUAD4         1       1       1       1       1\nENDDATA\n"),
    }
    import sys
    sys.path.insert(0, GOLDEN)
    import bdf_cases
    # CRLF under a continued card: the reference's loader aborts on it too
    bad["crlf_continuation"] = bdf_cases.crlf_continuation_deck()
    for key, text in bad.items():
        p = tmp_path / f"{key}.bdf"
        p.write_bytes(text.encode())
        with pytest.raises(capi.A2dsError):
            ml.scan_bdf_file(str(p))


def test_loader_assembler_inputs():
    """The shell-quad deck converts to Assembler inputs: Quad4 connectivity
    and the SPC entries as per-entry DOF masks and values."""
    ml = capi.MeshLoader()
    ml.scan_bdf_file(os.path.join(GOLDEN, "bdf_cyl_q4_8x16.bdf"))
    nodes, masks, v6 = ml.bc_masks()
    f = np.load(os.path.join(GOLDEN, "bdf_cyl_q4_8x16_lu.npz"))
    assert np.array_equal(nodes, f["bc_nodes"]) and np.array_equal(masks, f["bc_mask"])
    assert np.array_equal(v6, f["bc_vals"])
    mixed = capi.MeshLoader()
    mixed.scan_bdf_file(os.path.join(GOLDEN, "bdf_mixed.bdf"))
    with pytest.raises(capi.A2dsError):
        mixed.create_assembler()  # mixed element types


@pytest.mark.gpu
def test_bdf_cylinder_buckling_matches_reference():
    f = np.load(os.path.join(GOLDEN, "bdf_cyl_q4_8x16_lu.npz"))
    ml = capi.MeshLoader()
    ml.scan_bdf_file(os.path.join(GOLDEN, "bdf_cyl_q4_8x16.bdf"))
    a = ml.create_assembler()
    a.set_material(float(f["E"]), float(f["nu"]))
    a.set_thickness(f["thickness"][:1])
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    nev = 5
    b = capi.LinearBuckling(a, float(f["sigma"]), max_lanczos=120, num_eigvals=nev,
                            eig_tol=1e-12, lev_fill=1000000, precision=64, block_size=1)
    lam = b.solve(None)
    assert np.all(b.errors < 1e-8), b.errors
    # the load path comes from the prescribed end displacement alone
    assert np.abs(b.path).max() > 0
    ref = f["eigvals_dense"][:nev]
    assert np.max(np.abs(lam - ref) / np.abs(ref)) < 1e-8, (lam, ref)
    assert np.abs(b.path - f["path"]).max() / np.abs(f["path"]).max() < 1e-8
