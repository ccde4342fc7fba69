""".f5 output (TACSToFH5::writeToFile, src/io/TACSToFH5.cpp:126, through
TACSFH5File) against files the reference itself wrote (tests/golden/f5.npz,
oracle/ref/golden_gen.cpp f5 mode): byte-identical for a Quad4 and a Quad9
cylinder and a Quad9 stiffened panel (skin and blade webs) with two named
components, for the connectivity, node and
displacement output classes alone and together (CPU); with the load and
element classes (computed on the GPU) the layout is byte-identical and the
values agree to FP32 rounding (GPU)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from a2ds import capi

FLAGS = [capi.A2DS_F5_CONNECTIVITY | capi.A2DS_F5_NODES | capi.A2DS_F5_DISPLACEMENTS,
         capi.A2DS_F5_NODES, capi.A2DS_F5_DISPLACEMENTS, capi.A2DS_F5_CONNECTIVITY]


@pytest.mark.parametrize("mesh", ["q4", "q9", "panel"])
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
@pytest.mark.parametrize("flag", [capi.A2DS_F5_LOADS, 71, capi.A2DS_F5_STRAINS | capi.A2DS_F5_STRESSES,
                                  capi.A2DS_F5_EXTRAS, 127])
def test_f5_gpu_classes_match_reference(mesh, flag, tmp_path):
    """Loads (the GPU residual) and the element classes (strains, stresses
    and extras at every element node point, from the GPU element kernel):
    layout byte-identical, values to FP32 rounding of the reference's."""
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g[f"{mesh}__X"], g[f"{mesh}__conn"])
    a.set_material(70e9, 0.3)
    a.set_thickness([1e-2])
    a.set_yield_stress(270e6)
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
            # per column: FP32 rounding of values computed in a different
            # order (the columns span strains, stresses and failure values)
            d2 = zo[4]
            vo, vr = vo.reshape(-1, d2), vr.reshape(-1, d2)
            scale = np.maximum(np.abs(vr).max(axis=0), 1e-30)
            assert np.all(np.abs(vo - vr).max(axis=0) <= 1e-5 * scale), (
                np.abs(vo - vr).max(axis=0) / scale)


def test_f5_argument_errors(tmp_path):
    g = np.load(os.path.join(GOLDEN, "f5.npz"))
    a = capi.Assembler(g["q4__X"], g["q4__conn"])
    with pytest.raises(capi.A2dsError):  # an unknown output class bit
        capi.ToFH5(a, capi.A2DS_F5_NODES | 128).write_to_file(str(tmp_path / "x.f5"))
    with pytest.raises(capi.A2dsError):  # failure values without a yield stress
        capi.ToFH5(a, capi.A2DS_F5_EXTRAS).write_to_file(str(tmp_path / "x.f5"))
    with pytest.raises(capi.A2dsError):  # element classes before initialize()
        a.set_yield_stress(270e6)
        capi.ToFH5(a, capi.A2DS_F5_STRAINS).write_to_file(str(tmp_path / "x.f5"))
