""".f5 output (TACSToFH5::writeToFile, src/io/TACSToFH5.cpp:126, through
TACSFH5File) against files the reference itself wrote (tests/golden/f5.npz,
oracle/ref/golden_gen.cpp f5 mode): byte-identical for a Quad4 and a Quad9
mesh with two named components, for the connectivity, node and
displacement output classes alone and together."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from a2ds import capi

FLAGS = [capi.A2DS_F5_CONNECTIVITY | capi.A2DS_F5_NODES | capi.A2DS_F5_DISPLACEMENTS,
         capi.A2DS_F5_NODES, capi.A2DS_F5_DISPLACEMENTS, capi.A2DS_F5_CONNECTIVITY]


@pytest.mark.parametrize("mesh", ["q4", "q9"])
@pytest.mark.parametrize("flag", FLAGS)
def test_f5_bytes_match_reference(mesh, flag, tmp_path):
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g[f"{mesh}__X"], g[f"{mesh}__conn"])
    out = capi.ToFH5(a, flag, elem_component=g[f"{mesh}__comp"])
    out.set_component_name(0, "skin")
    out.set_component_name(1, "stiffener panel")
    path = tmp_path / "out.f5"
    out.write_to_file(str(path), g[f"{mesh}__vars"])
    assert path.read_bytes() == g[f"{mesh}__f5_{flag}"].tobytes()


def test_f5_rejects_element_output_classes(tmp_path):
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g["q4__X"], g["q4__conn"])
    strains = 8  # TACS_OUTPUT_STRAINS: element output classes are not written
    with pytest.raises(capi.A2dsError):
        capi.ToFH5(a, capi.A2DS_F5_NODES | strains).write_to_file(str(tmp_path / "x.f5"))
