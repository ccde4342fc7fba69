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


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    return cxx


def build_driver(tmp_path):
    lib = capi.load()  # builds the library if needed
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "mech_buckling")
    subprocess.run([_cxx(), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE,
                    DRIVER, "-L", libdir, "-la2ds_gpu", f"-Wl,-rpath,{libdir}", "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_alone(tmp_path):
    src = tmp_path / "only_header.cpp"
    src.write_text('#include "a2ds_tacs.hpp"\nint main() { return 0; }\n')
    subprocess.run([_cxx(), "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                    INCLUDE, str(src)], check=True, capture_output=True, text=True)


def test_driver_builds(tmp_path):
    assert os.path.exists(build_driver(tmp_path))


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
