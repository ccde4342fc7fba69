"""The C++ classes of include/a2ds_tacs.hpp (the reference's class names on
the buckling path over the C ABI) driven by tests/cpp/mech_buckling.cpp,
the call sequence of the reference's examples/cylinder-buckling/
mechBuckling.cpp.

* CPU: the header compiles on its own and the driver compiles and links
  against the built library with all warnings as errors.
* GPU: the driver reads the displacement-controlled cylinder deck
  (tests/golden/bdf_cyl_q4_8x16.bdf), solves for its lowest buckling loads
  and writes the first mode to .f5; the loads match the reference's
  TACSLinearBuckling solution of the same deck (a dense FP64 solve of its
  K and G, tests/golden/bdf_cyl_q4_8x16_lu.npz) to 1e-8.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO
from a2ds import capi

INCLUDE = os.path.join(REPO, "include")
DRIVER = os.path.join(REPO, "tests", "cpp", "mech_buckling.cpp")
SEQUENCE = os.path.join(REPO, "tests", "cpp", "assembler_sequence.cpp")


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    return cxx


def build_driver(tmp_path, src=DRIVER):
    lib = capi.load()  # builds the library if needed
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    subprocess.run([_cxx(), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE,
                    src, "-L", libdir, "-la2ds_gpu", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_alone(tmp_path):
    src = tmp_path / "only_header.cpp"
    src.write_text('#include "a2ds_tacs.hpp"\nint main() { return 0; }\n')
    subprocess.run([_cxx(), "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                    INCLUDE, str(src)], check=True, capture_output=True, text=True)


def test_driver_builds(tmp_path):
    assert os.path.exists(build_driver(tmp_path))
    assert os.path.exists(build_driver(tmp_path, SEQUENCE))


@pytest.mark.gpu
def test_reference_construction_sequence(tmp_path):
    """TACSAssembler(comm, 6, nodes, elements) + setElementConnectivity +
    setElements + addBCs + setNodes + initialize, then the buckling solve
    (loads within 1e-8 of a dense solve of the same mesh), checkEigenvector,
    a BCSRMat complete-LU factor object (one applyFactor leaves a relative
    residual ||K y - x|| / ||x|| below 1e-6: one FP64 LU solve of this thin
    shell's K, cond ~1e10, without refinement; measured 4e-8) and
    assembleJacobian(alpha = 2) (= 2 K off the Dirichlet rows)."""
    from a2ds import mesh as meshgen
    from test_gpu_solve import dense_buckling
    m = meshgen.cylinder(4, 8)
    d = tmp_path / "mesh"
    d.mkdir()
    np.array([m.num_nodes, m.num_elements, 4, m.bc_nodes.size], np.int32).tofile(d / "sizes.i32")
    np.ascontiguousarray(m.X, np.float64).tofile(d / "X.f64")
    np.ascontiguousarray(m.conn, np.int32).tofile(d / "conn.i32")
    np.ascontiguousarray(m.bc_nodes, np.int32).tofile(d / "bc_nodes.i32")
    np.ascontiguousarray(m.rhs, np.float64).tofile(d / "rhs.f64")
    np.array([m.E, m.nu, m.meta["t"]], np.float64).tofile(d / "params.f64")
    # dense truth of the same mesh through the Python classes
    a = capi.Assembler(m.X, m.conn)
    a.set_material(m.E, m.nu)
    a.set_thickness([m.meta["t"]])
    a.add_bcs(m.bc_nodes, m.bc_mask, m.bc_vals)
    a.initialize(capi.A2DS_TACS_AMD_ORDER)
    lam_cl = meshgen.classical_cylinder_load(m.E, m.nu, m.meta["t"], 1.0)
    b = capi.LinearBuckling(a, 0.3 * lam_cl, max_lanczos=120, num_eigvals=1, eig_tol=1e-12)
    b.solve(m.rhs)
    K, G = a.create_mat(), a.create_mat()
    a.assemble_mat_type(capi.A2DS_STIFFNESS_MATRIX, K)
    a.assemble_mat_type(capi.A2DS_GEOMETRIC_STIFFNESS_MATRIX, G, b.path)
    dense = dense_buckling(K.to_dense_nodes(), G.to_dense_nodes(), m.bc_nodes, m.bc_mask)
    nev = 4
    exe = build_driver(tmp_path, SEQUENCE)
    r = subprocess.run([exe, str(d), repr(0.9 * float(dense[0])), str(nev)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    lines = r.stdout.splitlines()
    lam = np.array([float(x.split()[2]) for x in lines if x.startswith("eig ")])
    assert lam.size == nev
    assert np.max(np.abs(lam - dense[:nev]) / np.abs(dense[:nev])) < 1e-8, (lam, dense[:nev])
    val = {x.split()[0]: float(x.split()[1]) for x in lines
           if x.split()[0] in ("check", "apply", "jac")}
    assert 0.0 <= val["check"] < 1e-6, r.stdout
    assert val["apply"] < 1e-6, r.stdout
    assert val["jac"] < 1e-14, r.stdout


@pytest.mark.gpu
def test_driver_matches_reference(tmp_path):
    exe = build_driver(tmp_path)
    f = np.load(os.path.join(GOLDEN, "bdf_cyl_q4_8x16_lu.npz"))
    out = str(tmp_path / "mode0.f5")
    nev = 5
    r = subprocess.run([exe, os.path.join(GOLDEN, "bdf_cyl_q4_8x16.bdf"), repr(float(f["E"])),
                        repr(float(f["nu"])), repr(float(f["thickness"][0])),
                        repr(float(f["sigma"])), str(nev), out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [line.split() for line in r.stdout.strip().splitlines()]
    lam = np.array([float(x[1]) for x in rows])
    err = np.array([float(x[2]) for x in rows])
    ref = f["eigvals_dense"][:nev]
    assert lam.size == nev and np.all(err < 1e-8), r.stdout
    assert np.max(np.abs(lam - ref) / np.abs(ref)) < 1e-8, (lam, ref)
    assert os.path.getsize(out) > 0
