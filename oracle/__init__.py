"""CPU restatement of the reference's buckling hot path -- TEST INFRASTRUCTURE.

This package is the checker the GB300 path is compared against and the timed
CPU baseline (bench.py's cpu_baseline and --impl reference legs).  Only
tests/, __graft_entry__.smoke() and bench.py may import it; the shipped
library never does.

The C sources in oracle/c/ restate the reference (sean-engelstad/a2d-shells)
function by function; they are pinned against fixtures generated by the
reference itself (tests/golden/, see tests/golden/make_golden.py and
oracle/ref/).  `load()` compiles them with gcc into oracle/_build/ on first
use (also on the GPU machine, where no prebuilt x86 binary survives).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = [os.path.join(HERE, "c", f) for f in sorted(os.listdir(os.path.join(HERE, "c")))
           if f.endswith(".c")]
_lock = threading.Lock()
_lib = None

P = ctypes.POINTER(ctypes.c_double)
PI = ctypes.POINTER(ctypes.c_int)


class Material(ctypes.Structure):
    """orc_material (oracle/c/shell_oracle.h)."""
    _fields_ = [(n, ctypes.c_double) for n in
                ["E", "nu", "t", "alpha", "temperature", "kcorr", "drill_reg", "t_offset"]]

    @classmethod
    def iso(cls, E, nu, t, alpha=0.0, temperature=0.0):
        return cls(E, nu, t, alpha, temperature, 5.0 / 6.0, 10.0, 0.0)


def build(force: bool = False) -> str:
    """Compile the oracle C sources (gcc, -O2, OpenMP) if they are newer than the library."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(HERE, "c", f) for f in os.listdir(os.path.join(HERE, "c"))
               if f.endswith(".h")]
    newest = max(os.path.getmtime(f) for f in SOURCES + headers)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-fopenmp", "-o", tmp] + \
            SOURCES + ["-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            _declare(_lib)
        return _lib


def _declare(lib):
    lib.orc_get_mat_type.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(Material), P, P, P]
    lib.orc_add_residual.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Material),
                                     P, P, P]
    lib.orc_add_jacobian.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Material),
                                     ctypes.c_double, P, P, P, P]


def _p(a):
    return a.ctypes.data_as(P)


STIFFNESS, MASS, GEOMETRIC = 0, 1, 2


def element_matrix(order, nonlinear, kind, mat: Material, X, vars_):
    """TACSShellElement::getMatType for one element (row-major (6nn)^2)."""
    lib = load()
    nv = 6 * order * order
    X = np.ascontiguousarray(X, dtype=np.float64)
    v = np.ascontiguousarray(vars_, dtype=np.float64)
    out = np.zeros((nv, nv))
    lib.orc_get_mat_type(order, int(nonlinear), kind, ctypes.byref(mat), _p(X), _p(v), _p(out))
    return out


def element_residual(order, nonlinear, mat: Material, X, vars_):
    lib = load()
    nv = 6 * order * order
    X = np.ascontiguousarray(X, dtype=np.float64)
    v = np.ascontiguousarray(vars_, dtype=np.float64)
    out = np.zeros(nv)
    lib.orc_add_residual(order, int(nonlinear), ctypes.byref(mat), _p(X), _p(v), _p(out))
    return out


def element_jacobian(order, nonlinear, mat: Material, X, vars_, alpha=1.0):
    lib = load()
    nv = 6 * order * order
    X = np.ascontiguousarray(X, dtype=np.float64)
    v = np.ascontiguousarray(vars_, dtype=np.float64)
    res = np.zeros(nv)
    J = np.zeros((nv, nv))
    lib.orc_add_jacobian(order, int(nonlinear), ctypes.byref(mat), alpha, _p(X), _p(v),
                         _p(res), _p(J))
    return res, J
