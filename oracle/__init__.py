"""CPU restatement of the reference's buckling hot path -- TEST INFRASTRUCTURE.

This package is the checker the GB300 path is compared against and the timed
CPU baseline (bench.py's cpu_baseline and --impl reference legs).  Only
tests/, __graft_entry__.smoke() and bench.py may import it; the shipped
library never does.

The C sources in oracle/c/ restate the reference (sean-engelstad/a2d-shells)
function by function; they are pinned against fixtures generated by the
reference itself (tests/golden/, see tests/golden/make_golden.py and
oracle/ref/).  `load()` compiles them with gcc into oracle/_build/ on first
use (on every machine, since a binary built on another architecture does
not run).
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
        cmd = ["gcc", "-O3", "-fPIC", "-shared", "-std=gnu99", "-fopenmp", "-o", tmp] + \
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


def element_xpt_inner_product(order, nonlinear, kind, mat: Material, X, vars_, psi, phi,
                              dh=1e-7):
    """d(sum_ij M[j][i] psi_i phi_j)/dX for one element (3 nn values):
    TACSElement::addMatXptSensInnerProduct (src/elements/TACSElement.cpp:
    434-507) in its real-mode form, second-order central differences with
    step dh in each coordinate."""
    X = np.array(X, dtype=np.float64).reshape(-1)
    psi = np.asarray(psi, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    out = np.zeros(X.size)
    for k in range(X.size):
        xt = X[k]
        X[k] = xt + dh
        p2 = phi @ element_matrix(order, nonlinear, kind, mat, X, vars_) @ psi
        X[k] = xt - dh
        p1 = phi @ element_matrix(order, nonlinear, kind, mat, X, vars_) @ psi
        X[k] = xt
        out[k] = 0.5 * (p2 - p1) / dh
    return out


def element_sv_inner_product(order, nonlinear, kind, mat: Material, X, vars_, psi, phi,
                             dh=1e-7):
    """d(sum_ij M[j][i] psi_i phi_j)/d(vars) for one element (6 nn values):
    TACSElement::getMatSVSensInnerProduct (src/elements/TACSElement.cpp:
    509-581), real-mode central differences with step dh."""
    v = np.array(vars_, dtype=np.float64).reshape(-1)
    psi = np.asarray(psi, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    out = np.zeros(v.size)
    for k in range(v.size):
        vt = v[k]
        v[k] = vt + dh
        p2 = phi @ element_matrix(order, nonlinear, kind, mat, X, v) @ psi
        v[k] = vt - dh
        p1 = phi @ element_matrix(order, nonlinear, kind, mat, X, v) @ psi
        v[k] = vt
        out[k] = 0.5 * (p2 - p1) / dh
    return out


def element_adjres_xpt_product(order, nonlinear, mat: Material, X, vars_, psi, dh=1e-7):
    """psi^T dR/dX for one element (3 nn values): TACSElement::
    addAdjResXptProduct (src/elements/TACSElement.cpp:270-330), real-mode
    central differences with step dh (psi times the residual difference,
    divided by 2 dh)."""
    X = np.array(X, dtype=np.float64).reshape(-1)
    psi = np.asarray(psi, dtype=np.float64)
    out = np.zeros(X.size)
    for k in range(X.size):
        xt = X[k]
        X[k] = xt + dh
        r2 = element_residual(order, nonlinear, mat, X, vars_)
        X[k] = xt - dh
        r1 = element_residual(order, nonlinear, mat, X, vars_)
        X[k] = xt
        out[k] = np.sum(psi * (r2 - r1) / (2.0 * dh))
    return out


# ------------------------------------------------------------- solve path
def _declare_solver(lib):
    lib.orc_assemble.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(Material), ctypes.c_int, ctypes.c_int, PI, PI,
                                 P, P, P, PI, PI, PI, P]
    lib.orc_apply_bcs.argtypes = [PI, PI, P, ctypes.c_int, PI, PI]
    lib.orc_spmv.argtypes = [ctypes.c_int, PI, PI, P, P, P]
    lib.orc_factor_fill.argtypes = [ctypes.c_int, PI, PI, P, PI, PI, P]
    lib.orc_factor.argtypes = [ctypes.c_int, PI, PI, PI, P]
    lib.orc_factor.restype = ctypes.c_int
    lib.orc_apply_factor.argtypes = [ctypes.c_int, PI, PI, PI, P, P, P]
    lib.orc_gmres.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                              ctypes.c_double, P, P]
    lib.orc_gmres.restype = ctypes.c_int
    lib.orc_lanczos.argtypes = [ctypes.c_void_p, ctypes.c_int, PI, PI, P, ctypes.c_double,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_int, PI, PI, ctypes.c_uint, ctypes.c_int, P]
    lib.orc_lanczos.restype = ctypes.c_int


class _System(ctypes.Structure):
    """orc_system (oracle/c/solver_oracle.c)"""
    _fields_ = [("n", ctypes.c_int), ("rowp", PI), ("cols", PI), ("A", P),
                ("frowp", PI), ("fcols", PI), ("fdiag", PI), ("F", P)]


def _pi(a):
    return a.ctypes.data_as(PI)


def assemble(mesh, kind, perm, rowp, cols, vars_=None, nonlinear=False, bc_rows=None,
             bc_masks=None):
    """TACSAssembler::assembleMatType on the CPU: BCSR values in the matrix
    ordering given by perm (row i <-> node perm[i]) and pattern rowp/cols."""
    lib = load()
    _declare_solver(lib)
    n = perm.size
    iperm = np.empty(n, np.int32)
    iperm[perm] = np.arange(n, dtype=np.int32)
    conn = np.ascontiguousarray(mesh.conn, np.int32)
    conn_rows = np.ascontiguousarray(iperm[conn], np.int32)
    X = np.ascontiguousarray(mesh.X, np.float64)
    v = None if vars_ is None else np.ascontiguousarray(vars_, np.float64)
    tv = np.ascontiguousarray(mesh.thickness, np.float64)  # one group per element
    tg = np.arange(mesh.num_elements, dtype=np.int32)
    rowp = np.ascontiguousarray(rowp, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.zeros((cols.size, 6, 6))
    m = Material.iso(mesh.E, mesh.nu, 1.0)
    lib.orc_assemble(mesh.order, int(nonlinear), kind, ctypes.byref(m), n, mesh.num_elements,
                     _pi(conn), _pi(conn_rows), _p(X), None if v is None else _p(v), _p(tv),
                     _pi(tg), _pi(rowp), _pi(cols), _p(vals))
    if bc_rows is not None and len(bc_rows):
        br = np.ascontiguousarray(bc_rows, np.int32)
        bm = np.ascontiguousarray(bc_masks, np.int32)
        lib.orc_apply_bcs(_pi(rowp), _pi(cols), _p(vals), br.size, _pi(br), _pi(bm))
    return vals


def factor(rowp, cols, vals, frowp, fcols, fdiag):
    """BCSRMatFactor6 on the CPU (diagonal blocks inverted in place)."""
    lib = load()
    _declare_solver(lib)
    n = rowp.size - 1
    F = np.zeros((fcols.size, 6, 6))
    args = [np.ascontiguousarray(a, np.int32) for a in (rowp, cols, frowp, fcols, fdiag)]
    lib.orc_factor_fill(n, _pi(args[0]), _pi(args[1]), _p(np.ascontiguousarray(vals)),
                        _pi(args[2]), _pi(args[3]), _p(F))
    rc = lib.orc_factor(n, _pi(args[2]), _pi(args[3]), _pi(args[4]), _p(F))
    if rc:
        raise RuntimeError(f"singular diagonal block in row {rc - 1}")
    return F


def gmres(rowp, cols, A, frowp, fcols, fdiag, F, m, nrestart, rtol, atol, b):
    """GMRES::solve (src/bpmat/KSM.cpp:785-970) on the CPU: right
    preconditioned by the factor F, zero initial guess.  Returns (x, iterations)."""
    lib = load()
    _declare_solver(lib)
    n = rowp.size - 1
    args = [np.ascontiguousarray(v, np.int32) for v in (rowp, cols, frowp, fcols, fdiag)]
    A = np.ascontiguousarray(A, np.float64)
    F = np.ascontiguousarray(F, np.float64)
    sysA = _System(n, _pi(args[0]), _pi(args[1]), _p(A), _pi(args[2]), _pi(args[3]),
                   _pi(args[4]), _p(F))
    b = np.ascontiguousarray(b, np.float64).ravel()
    x = np.zeros_like(b)
    it = lib.orc_gmres(ctypes.byref(sysA), int(m), int(nrestart), float(rtol), float(atol),
                       _p(b), _p(x))
    return x, it


class CpuBuckling:
    """The reference's buckling path on the CPU (TACSLinearBuckling::solve
    with a TACSSchurPc factor of K and GMRES on K + sigma G), timed phase by
    phase.  Pattern, ordering and factor pattern are inputs (integer host
    work, checked bit-exact against the reference separately)."""

    def __init__(self, mesh, perm, rowp, cols, frowp, fcols, fdiag, bc_rows, bc_masks):
        self.mesh, self.perm = mesh, np.ascontiguousarray(perm, np.int32)
        self.rowp, self.cols = np.ascontiguousarray(rowp, np.int32), np.ascontiguousarray(cols, np.int32)
        self.frowp, self.fcols = np.ascontiguousarray(frowp, np.int32), np.ascontiguousarray(fcols, np.int32)
        self.fdiag = np.ascontiguousarray(fdiag, np.int32)
        self.bc_rows = np.ascontiguousarray(bc_rows, np.int32)
        self.bc_masks = np.ascontiguousarray(bc_masks, np.int32)
        self.times = {}

    def _to_rows(self, v):
        return np.ascontiguousarray(np.asarray(v).reshape(-1, 6)[self.perm]).ravel()

    def _from_rows(self, v):
        out = np.empty_like(v.reshape(-1, 6))
        out[self.perm] = v.reshape(-1, 6)
        return out

    def solve(self, sigma, rhs, lanczos_iters=10, num_eig=10, gm_m=10, gm_restarts=15,
              gm_tol=1e-12, seed=0):
        import time
        lib = load()
        _declare_solver(lib)
        n = self.rowp.size - 1
        t = self.times
        t0 = time.perf_counter()
        K = assemble(self.mesh, STIFFNESS, self.perm, self.rowp, self.cols, None, False,
                     self.bc_rows, self.bc_masks)
        t["assemble_k"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        F = factor(self.rowp, self.cols, K, self.frowp, self.fcols, self.fdiag)
        t["factor"] = time.perf_counter() - t0
        # load path: GMRES on K (aux = K at this point), pc = factor of K
        t0 = time.perf_counter()
        b = self._to_rows(rhs)
        for r, mk in zip(self.bc_rows, self.bc_masks):
            for k in range(6):
                if mk >> k & 1:
                    b[6 * r + k] = 0.0
        path = np.zeros_like(b)
        sysK = _System(n, _pi(self.rowp), _pi(self.cols), _p(K), _pi(self.frowp),
                       _pi(self.fcols), _pi(self.fdiag), _p(F))
        lib.orc_gmres(ctypes.byref(sysK), gm_m, gm_restarts, gm_tol, gm_tol, _p(b), _p(path))
        t["path"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        G = assemble(self.mesh, GEOMETRIC, self.perm, self.rowp, self.cols,
                     self._from_rows(path), False, self.bc_rows, self.bc_masks)
        t["assemble_g"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        A = np.ascontiguousarray(K + sigma * G)
        lib.orc_apply_bcs(_pi(self.rowp), _pi(self.cols), _p(A), self.bc_rows.size,
                          _pi(self.bc_rows), _pi(self.bc_masks))
        sysA = _System(n, _pi(self.rowp), _pi(self.cols), _p(A), _pi(self.frowp),
                       _pi(self.fcols), _pi(self.fdiag), _p(F))
        lam = np.zeros(num_eig)
        gm = lib.orc_lanczos(ctypes.byref(sysA), n, _pi(self.rowp), _pi(self.cols), _p(K),
                             sigma, lanczos_iters, gm_m, gm_restarts, gm_tol, self.bc_rows.size,
                             _pi(self.bc_rows), _pi(self.bc_masks), seed, num_eig, _p(lam))
        t["lanczos"] = time.perf_counter() - t0
        t["gmres_iters"] = gm
        self.path = self._from_rows(path)
        self.eigvals = lam
        return lam


# ------------------------------------------- multi-threaded CPU solve
def _declare_par(lib):
    lib.orc_nd_order.argtypes = [ctypes.c_int, PI, PI, P, ctypes.c_int, PI]
    lib.orc_symbolic_lu.argtypes = [ctypes.c_int, PI, PI, PI, PI]
    lib.orc_symbolic_lu.restype = ctypes.c_longlong
    lib.orc_factor_levels.argtypes = [ctypes.c_int, PI, PI, PI, ctypes.c_int, PI, PI]
    lib.orc_factor_levels.restype = ctypes.c_int
    lib.orc_factor_par.argtypes = [ctypes.c_int, PI, PI, PI, ctypes.c_int, PI, PI, P]
    lib.orc_factor_par.restype = ctypes.c_int
    lib.orc_apply_factor_par.argtypes = [ctypes.c_int, PI, PI, PI, P, ctypes.c_int, PI, PI,
                                         ctypes.c_int, PI, PI, ctypes.c_int, P, P]
    lib.orc_spmm.argtypes = [ctypes.c_int, PI, PI, P, ctypes.c_int, P, P, P]
    lib.omp_get_max_threads.restype = ctypes.c_int


def node_graph(conn, nn):
    """Node-to-node CSR (with the diagonal, sorted) of an element mesh."""
    conn = np.asarray(conn, np.int64)
    npe = conn.shape[1]
    a = np.repeat(conn, npe, axis=1).ravel()
    b = np.tile(conn, (1, npe)).ravel()
    key = np.unique(a * nn + b)
    r, c = key // nn, key % nn
    rowp = np.zeros(nn + 1, np.int32)
    np.add.at(rowp, r + 1, 1)
    return np.cumsum(rowp).astype(np.int32), c.astype(np.int32)


class CpuPlan:
    """Host set-up of the multi-threaded CPU solve: nested-dissection
    ordering (cpu_parallel.c), the BCSR pattern in that ordering, the
    complete-LU pattern from the elimination tree and the dependency levels
    of its triangular solves.  Needs nothing but the oracle library."""

    def __init__(self, mesh):
        lib = load()
        _declare_solver(lib)
        _declare_par(lib)
        self.lib = lib
        nn = mesh.num_nodes
        grp, grc = node_graph(mesh.conn, nn)
        perm = np.empty(nn, np.int32)
        X = np.ascontiguousarray(mesh.X, np.float64)
        lib.orc_nd_order(nn, _pi(grp), _pi(grc), _p(X), 64, _pi(perm))
        iperm = np.empty(nn, np.int32)
        iperm[perm] = np.arange(nn, dtype=np.int32)
        # pattern in the row ordering
        r = iperm[np.repeat(np.arange(nn), np.diff(grp))].astype(np.int64)
        c = iperm[grc].astype(np.int64)
        key = np.unique(r * nn + c)
        rowp = np.zeros(nn + 1, np.int32)
        np.add.at(rowp, (key // nn) + 1, 1)
        self.perm, self.iperm = perm, iperm
        self.rowp = np.cumsum(rowp).astype(np.int32)
        self.cols = (key % nn).astype(np.int32)
        nf = lib.orc_symbolic_lu(nn, _pi(self.rowp), _pi(self.cols), None, None)
        self.frowp = np.zeros(nn + 1, np.int32)
        self.fcols = np.zeros(nf, np.int32)
        lib.orc_symbolic_lu(nn, _pi(self.rowp), _pi(self.cols), _pi(self.frowp), _pi(self.fcols))
        self.fdiag = np.empty(nn, np.int32)
        for i in range(0, nn, 65536):  # position of the diagonal in each row
            j = np.arange(i, min(nn, i + 65536))
            lens = self.frowp[j + 1] - self.frowp[j]
            rows = np.repeat(j, lens)
            pos = np.arange(self.frowp[i], self.frowp[j[-1] + 1])
            hit = self.fcols[pos] == rows
            self.fdiag[rows[hit]] = pos[hit]
        self.levels = {}
        for upper in (0, 1):
            nl = lib.orc_factor_levels(nn, _pi(self.frowp), _pi(self.fcols), _pi(self.fdiag),
                                       upper, None, None)
            ptr = np.zeros(nl + 1, np.int32)
            rows = np.zeros(nn, np.int32)
            lib.orc_factor_levels(nn, _pi(self.frowp), _pi(self.fcols), _pi(self.fdiag), upper,
                                  _pi(ptr), _pi(rows))
            self.levels[upper] = (nl, ptr, rows)
        self.n = nn
        self.bc_rows = iperm[mesh.bc_nodes].astype(np.int32)
        self.bc_masks = np.ascontiguousarray(mesh.bc_mask, np.int32)
        mask = np.zeros((nn, 6), bool)
        for rr, mk in zip(self.bc_rows, self.bc_masks):
            for k in range(6):
                if mk >> k & 1:
                    mask[rr, k] = True
        self.bc_dofs = mask.ravel()

    @property
    def threads(self):
        return int(self.lib.omp_get_max_threads())

    def factor(self, vals):
        lib, n = self.lib, self.n
        F = np.zeros((self.fcols.size, 6, 6))
        lib.orc_factor_fill(n, _pi(self.rowp), _pi(self.cols), _p(np.ascontiguousarray(vals)),
                            _pi(self.frowp), _pi(self.fcols), _p(F))
        nl, ptr, rows = self.levels[0]
        rc = lib.orc_factor_par(n, _pi(self.frowp), _pi(self.fcols), _pi(self.fdiag), nl,
                                _pi(ptr), _pi(rows), _p(F))
        if rc:
            raise RuntimeError(f"singular diagonal block in row {rc - 1}")
        return F

    def apply(self, F, X):
        """(LU)^{-1} X for X of shape (6 n, p), row-major (row, dof, rhs)."""
        X = np.ascontiguousarray(X)
        p = X.shape[1] if X.ndim == 2 else 1
        Y = np.empty_like(X)
        (nlo, plo, rlo), (nup, pup, rup) = self.levels[0], self.levels[1]
        self.lib.orc_apply_factor_par(self.n, _pi(self.frowp), _pi(self.fcols), _pi(self.fdiag),
                                      _p(F), nlo, _pi(plo), _pi(rlo), nup, _pi(pup), _pi(rup), p,
                                      _p(X), _p(Y))
        return Y

    def spmm(self, A, X, B=None):
        X = np.ascontiguousarray(X)
        p = X.shape[1] if X.ndim == 2 else 1
        Y = np.empty_like(X)
        self.lib.orc_spmm(self.n, _pi(self.rowp), _pi(self.cols), _p(A), p, _p(X),
                          None if B is None else _p(np.ascontiguousarray(B)), _p(Y))
        return Y

    def assemble(self, mesh, kind, path_nodes=None):
        return assemble(mesh, kind, self.perm, self.rowp, self.cols, path_nodes, False,
                        self.bc_rows, self.bc_masks)

    def refined_solve(self, A, F, X, rtol, max_steps):
        Y = self.apply(F, X)
        xn = np.linalg.norm(X, axis=0)
        for _ in range(max_steps):
            R = self.spmm(A, Y, X)
            if np.all(np.linalg.norm(R, axis=0) <= rtol * xn):
                break
            Y += self.apply(F, R)
        return Y


def cpu_buckling_solve(mesh, plan: CpuPlan, sigma, neig=10, block=4, max_lanczos=200,
                       eig_tol=1e-8, seed=0):
    """The buckling solve on the host cores with the reference's numerics
    (element assembly, IKJ block LU, block triangular solves, SpMV) in the
    scheme of the GPU's all-FP64 solve: K at the zero state, its factor and
    the load path with FP64 refinement, G along the path, the factor of
    K + sigma G, and block shift-invert Lanczos (block `block`, two
    classical Gram-Schmidt passes in the K inner product, Cholesky-QR twice,
    Ritz convergence ||B_j y_j|| <= eig_tol |mu|).  Returns (eigenvalues,
    phase times, Lanczos vectors)."""
    import time
    t = {}
    n6 = 6 * plan.n
    lib = plan.lib
    t0 = time.perf_counter()
    K = plan.assemble(mesh, STIFFNESS)
    t["assemble_k"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    FK = plan.factor(K)
    t["factor_k"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = np.zeros((plan.n, 6))
    b[:] = mesh.rhs[plan.perm]
    for rr, mk in zip(plan.bc_rows, plan.bc_masks):
        for k in range(6):
            if mk >> k & 1:
                b[rr, k] = 0.0
    u = plan.refined_solve(K, FK, b.reshape(n6, 1), 1e-13, 4)
    path = np.empty((plan.n, 6))
    path[plan.perm] = u.reshape(plan.n, 6)
    t["path"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    G = plan.assemble(mesh, GEOMETRIC, path)
    t["assemble_g"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    A = np.ascontiguousarray(K + sigma * G)
    lib.orc_apply_bcs(_pi(plan.rowp), _pi(plan.cols), _p(A), plan.bc_rows.size,
                      _pi(plan.bc_rows), _pi(plan.bc_masks))
    FA = plan.factor(A)
    t["factor_a"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    p = block
    rng = np.random.default_rng(seed)
    bcd = plan.bc_dofs

    def korth(W, KW):
        for _ in range(2):
            M = W.T @ KW
            M = 0.5 * (M + M.T)
            R = np.linalg.cholesky(M).T
            Ri = np.linalg.inv(R)
            W[:] = W @ Ri
            KW[:] = KW @ Ri
            yield R

    def cholqr2(W, KW):
        Rs = list(korth(W, KW))
        return Rs[1] @ Rs[0]

    Q0 = rng.uniform(-1, 1, (n6, p))
    Q0[bcd] = 0.0
    Q, KQ = [Q0], [plan.spmm(K, Q0)]
    cholqr2(Q[0], KQ[0])
    nbmax = max_lanczos // p
    T = np.zeros(((nbmax + 1) * p, (nbmax + 1) * p))
    lam_of = lambda mu: -mu * sigma / (1.0 - mu)
    rtol = max(1e-12, min(1e-9, 0.1 * eig_tol))
    lam = None
    for j in range(nbmax):
        W = plan.refined_solve(A, FA, KQ[j], rtol, 2)
        W[bcd] = 0.0
        Qs = np.stack(Q)          # (j+1, n6, p)
        KQs = np.stack(KQ)
        H1 = np.einsum("bnc,nd->bcd", KQs, W)
        W -= np.einsum("bnc,bcd->nd", Qs, H1)
        H2 = np.einsum("bnc,nd->bcd", KQs, W)
        W -= np.einsum("bnc,bcd->nd", Qs, H2)
        H = H1 + H2
        KW = plan.spmm(K, W)
        B = cholqr2(W, KW)
        D = 0.5 * (H[j] + H[j].T)
        T[j * p:(j + 1) * p, j * p:(j + 1) * p] = D
        T[(j + 1) * p:(j + 2) * p, j * p:(j + 1) * p] = B
        T[j * p:(j + 1) * p, (j + 1) * p:(j + 2) * p] = B.T
        Q.append(W)
        KQ.append(KW)
        md = (j + 1) * p
        if md < neig:
            continue
        mu, V = np.linalg.eigh(T[:md, :md])
        order = np.argsort(np.abs(lam_of(mu)))[:neig]
        est = np.linalg.norm(B @ V[j * p:(j + 1) * p, order], axis=0)
        lam = lam_of(mu[order])
        if np.all(est <= eig_tol * np.abs(mu[order])):
            break
    t["lanczos"] = time.perf_counter() - t0
    return lam, t, (j + 1) * p
