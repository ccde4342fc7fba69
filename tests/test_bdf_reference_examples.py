"""The BDF loader on the reference's own example decks
(examples/cylinder-buckling/mech-cylinder.bdf and therm-cylinder.bdf: 3,300
GRID, 3,200 CQUAD4, SPC with an enforced end displacement) against the
reference's TACSMeshLoader run on the same files (oracle/_ref/golden_gen,
built from the reference sources).  Both the decks and the reference build
exist only where the reference tree is present; elsewhere the test is
skipped (the committed synthetic decks cover the loader everywhere)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO
from a2ds import capi

# the reference tree: A2DS_REFERENCE, else a checkout beside this repository
REFERENCE_TREE = (os.environ.get("A2DS_REFERENCE")
                  or os.path.join(os.path.dirname(REPO), "reference"))
DECKS = os.path.join(REFERENCE_TREE, "examples", "cylinder-buckling")
GOLDEN_GEN = os.path.join(REPO, "oracle", "_ref", "golden_gen")


@pytest.mark.parametrize("deck", ["mech-cylinder.bdf", "therm-cylinder.bdf"])
def test_loader_matches_reference_on_its_example_decks(deck):
    path = os.path.join(DECKS, deck)
    if not (os.path.exists(path) and os.access(GOLDEN_GEN, os.X_OK)):
        pytest.skip("reference tree or reference build not present")
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([GOLDEN_GEN, "bdf", path, d], check=True, capture_output=True)
        g = {f[:-4]: np.load(os.path.join(d, f)) for f in os.listdir(d) if f.endswith(".npy")}
    ml = capi.MeshLoader()
    ml.scan_bdf_file(path)
    fail, nn, ne, nbcs, ncomp = g["sizes"]
    assert fail == 0
    assert (ml.get_num_nodes(), ml.get_num_elements(), ml.get_num_components()) == (nn, ne, ncomp)
    assert (nn, ne) == (3300, 3200)
    ptr, conn, comp, X = ml.get_connectivity()
    assert np.array_equal(ptr, g["elem_node_ptr"])
    assert np.array_equal(conn, g["elem_node_conn"])
    assert np.array_equal(comp, g["elem_component"])
    assert np.array_equal(X, g["Xpts"])
    nodes, var, bptr, vals = ml.get_bcs()
    assert np.array_equal(nodes, g["bc_nodes"]) and np.array_equal(bptr, g["bc_ptr"])
    assert np.array_equal(var, g["bc_vars"]) and np.array_equal(vals, g["bc_vals"])
    names = [bytes(r).rstrip(b"\0").decode() for r in g["names"]]
    assert [ml.get_element_descript(c) for c in range(ncomp)] == names[:ncomp]
    assert [ml.get_component_descript(c) for c in range(ncomp)] == names[ncomp:]
    # the deck converts to the shell assembler's inputs (Quad4, SPC masks)
    a = ml.create_assembler()
    assert a.num_nodes == nn and a.num_elements == ne
