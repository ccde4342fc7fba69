""".f5 output (TACSToFH5::writeToFile, src/io/TACSToFH5.cpp:126, through
TACSFH5File) against files the reference itself wrote (tests/golden/f5.npz,
oracle/ref/golden_gen.cpp f5 mode): byte-identical for a Quad4 and a Quad9
mesh with two named components, for the connectivity, node and
displacement output classes alone and together (CPU); with the load class
(the residual assembled on the GPU) the layout is byte-identical and the
values agree to FP32 rounding (GPU)."""
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


def f5_zones(b):
    """(header bytes, [(zone header bytes, data bytes, type, dim1, dim2)])"""
    import struct
    n = struct.unpack_from("i", b, 0)[0]
    off = 4
    for _ in range(n):
        off += 4 + struct.unpack_from("i", b, off)[0]
    head, zones = b[:off], []
    while off < len(b):
        t, d1, d2, lz, lv = struct.unpack_from("5i", b, off)
        h0 = off
        off += 20 + lz + lv
        zones.append((b[h0:off], b[off:off + 4 * d1 * d2], t, d1, d2))
        off += 4 * d1 * d2
    return head, zones


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", ["q4", "q9"])
@pytest.mark.parametrize("flag", [capi.A2DS_F5_LOADS, 71])
def test_f5_loads_match_reference(mesh, flag, tmp_path):
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g[f"{mesh}__X"], g[f"{mesh}__conn"])
    a.set_material(70e9, 0.3)
    a.set_thickness([1e-2])
    a.initialize()
    out = capi.ToFH5(a, flag, elem_component=g[f"{mesh}__comp"])
    out.set_component_name(0, "skin")
    out.set_component_name(1, "stiffener panel")
    path = tmp_path / "out.f5"
    out.write_to_file(str(path), g[f"{mesh}__vars"])
    ours, ref = f5_zones(path.read_bytes()), f5_zones(g[f"{mesh}__f5_{flag}"].tobytes())
    assert ours[0] == ref[0] and len(ours[1]) == len(ref[1])
    for zo, zr in zip(ours[1], ref[1]):
        assert zo[0] == zr[0]  # zone header and names
        if zo[2] == 0:
            assert zo[1] == zr[1]  # integer zones
        else:
            vo = np.frombuffer(zo[1], np.float32).astype(np.float64)
            vr = np.frombuffer(zr[1], np.float32).astype(np.float64)
            assert np.abs(vo - vr).max() <= 1e-6 * np.abs(vr).max()


def test_f5_rejects_element_output_classes(tmp_path):
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g["q4__X"], g["q4__conn"])
    strains = 8  # TACS_OUTPUT_STRAINS: element output classes are not written
    with pytest.raises(capi.A2dsError):
        capi.ToFH5(a, capi.A2DS_F5_NODES | strains).write_to_file(str(tmp_path / "x.f5"))
