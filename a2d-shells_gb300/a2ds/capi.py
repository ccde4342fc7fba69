"""ctypes binding of the C ABI in include/a2ds.h, plus thin Python classes
that mirror the reference's call surface for this path:

  Assembler        TACSAssembler (src/TACSAssembler.h:59): mesh, material,
                   Dirichlet conditions, initialize, assembleMatType,
                   assembleRes, assembleJacobian
  BCSRMat          TACSSchurMat / BCSRMat (src/bpmat/BCSRMat.h:34): getArrays,
                   mult, copyValues, axpy, applyBCs
  SchurPc          TACSSchurPc (src/bpmat/TACSSchurMat.h:148): ILU(k) factor
  LinearBuckling   TACSLinearBuckling (src/TACSBuckling.h:43)

All arrays are numpy; every call goes to the GB300 library and raises
A2dsError on a non-zero status.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "liba2ds_gpu.so")

A2DS_STIFFNESS_MATRIX = 0
A2DS_GEOMETRIC_STIFFNESS_MATRIX = 2
A2DS_NATURAL_ORDER = 0
A2DS_RCM_ORDER = 1
A2DS_AMD_ORDER = 2
A2DS_ND_ORDER = 3
A2DS_TACS_AMD_ORDER = 4
A2DS_MULTICOLOR_ORDER = 5
A2DS_SCATTER_ATOMIC = 0
A2DS_SCATTER_COLORED = 1

ERRORS = {1: "A2DS_ERR_ARG", 2: "A2DS_ERR_STATE", 3: "A2DS_ERR_CUDA", 4: "A2DS_ERR_NOMEM",
          5: "A2DS_ERR_SINGULAR", 6: "A2DS_ERR_NOCONV", 7: "A2DS_ERR_BREAKDOWN",
          8: "A2DS_ERR_NUMERIC"}

# Every entry point of include/a2ds.h
EXPORTS = [
    "a2ds_last_error", "a2ds_device_count", "a2ds_mesh_create", "a2ds_mesh_destroy",
    "a2ds_mesh_set_material", "a2ds_mesh_set_yield_stress", "a2ds_mesh_set_thickness",
    "a2ds_mesh_add_bcs",
    "a2ds_mesh_plan", "a2ds_mesh_get_pattern", "a2ds_mesh_ilu_pattern",
    "a2ds_mesh_initialize", "a2ds_mesh_get_ordering", "a2ds_mesh_node_csr",
    "a2ds_bcsr_create", "a2ds_bcsr_destroy", "a2ds_bcsr_get", "a2ds_bcsr_set_values",
    "a2ds_assemble_mat", "a2ds_assemble_mat_ex", "a2ds_assemble_res", "a2ds_assemble_jacobian",
    "a2ds_add_mat_xpt_sens_inner_product", "a2ds_add_adjoint_res_xpt_sens_product",
    "a2ds_add_mat_dv_sens_inner_product", "a2ds_newton_preload", "a2ds_preload_buckling",
    "a2ds_preload_xpt_sens",
    "a2ds_eval_mat_sv_sens_inner_product", "a2ds_eig_sens_xpts",
    "a2ds_bcsr_mult", "a2ds_bcsr_mult_rows", "a2ds_bcsr_mult_rows_noalloc", "a2ds_bcsr_copy", "a2ds_bcsr_axpy",
    "a2ds_bcsr_time_mult", "a2ds_bcsr_time_mult_df",
    "a2ds_bcsr_apply_bcs", "a2ds_pc_create", "a2ds_pc_destroy", "a2ds_pc_factor",
    "a2ds_pc_apply", "a2ds_pc_apply_multi", "a2ds_pc_get", "a2ds_gmres_solve",
    "a2ds_fgmres_solve", "a2ds_buckling_default_opts", "a2ds_buckling_solve",
    "a2ds_buckling_stats", "a2ds_eig_sens_thickness", "a2ds_eigen_shift_invert",
    "a2ds_bdf_scan", "a2ds_bdf_destroy", "a2ds_bdf_get_sizes", "a2ds_bdf_get_connectivity",
    "a2ds_bdf_get_bcs", "a2ds_bdf_get_element_descript", "a2ds_bdf_get_component_descript",
    "a2ds_write_f5",
]


class A2dsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class BucklingOpts(ctypes.Structure):
    """a2ds_buckling_opts"""
    _fields_ = [("sigma", ctypes.c_double), ("max_lanczos", ctypes.c_int),
                ("num_eigvals", ctypes.c_int), ("eig_tol", ctypes.c_double),
                ("lev_fill", ctypes.c_int), ("gmres_m", ctypes.c_int),
                ("gmres_restarts", ctypes.c_int), ("gmres_rtol", ctypes.c_double),
                ("gmres_atol", ctypes.c_double), ("precision", ctypes.c_int),
                ("seed", ctypes.c_int), ("block_size", ctypes.c_int)]


_lib = None

P_D = ctypes.POINTER(ctypes.c_double)
P_I = ctypes.POINTER(ctypes.c_int)
VP = ctypes.c_void_p


def load(build: bool = False):
    """Load liba2ds_gpu.so (building it first when asked or when missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if build or not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("a2ds_build", os.path.join(PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.a2ds_last_error.restype = ctypes.c_char_p
    lib.a2ds_device_count.restype = ctypes.c_int
    lib.a2ds_mesh_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P_I, P_D,
                                     ctypes.c_int, ctypes.POINTER(VP)]
    lib.a2ds_mesh_destroy.argtypes = [VP]
    lib.a2ds_mesh_set_material.argtypes = [VP, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double]
    lib.a2ds_mesh_set_thickness.argtypes = [VP, ctypes.c_int, P_D, P_I]
    lib.a2ds_mesh_set_yield_stress.argtypes = [VP, ctypes.c_double]
    lib.a2ds_mesh_add_bcs.argtypes = [VP, ctypes.c_int, P_I, P_I, P_D]
    lib.a2ds_mesh_initialize.argtypes = [VP, ctypes.c_int]
    lib.a2ds_mesh_plan.argtypes = [VP, ctypes.c_int]
    lib.a2ds_mesh_get_pattern.argtypes = [VP, P_I, P_I, P_I]
    lib.a2ds_mesh_ilu_pattern.argtypes = [VP, ctypes.c_int, P_I, P_I, P_I]
    lib.a2ds_mesh_get_ordering.argtypes = [VP, P_I]
    lib.a2ds_mesh_node_csr.argtypes = [VP, ctypes.c_int, P_I, P_I, P_I]
    lib.a2ds_bcsr_create.argtypes = [VP, ctypes.POINTER(VP)]
    lib.a2ds_bcsr_destroy.argtypes = [VP]
    lib.a2ds_bcsr_get.argtypes = [VP, P_I, P_I, P_I, P_I, P_D]
    lib.a2ds_bcsr_set_values.argtypes = [VP, P_D]
    lib.a2ds_assemble_mat.argtypes = [VP, ctypes.c_int, P_D, VP]
    lib.a2ds_assemble_mat_ex.argtypes = [VP, ctypes.c_int, P_D, VP, ctypes.c_int]
    lib.a2ds_assemble_res.argtypes = [VP, P_D, P_D]
    lib.a2ds_assemble_jacobian.argtypes = [VP, P_D, P_D, VP]
    lib.a2ds_bcsr_mult.argtypes = [VP, P_D, P_D]
    lib.a2ds_bcsr_mult_rows.argtypes = [VP, P_D, P_D]
    lib.a2ds_bcsr_mult_rows_noalloc.argtypes = [VP, P_D, P_D]
    lib.a2ds_bcsr_copy.argtypes = [VP, VP]
    lib.a2ds_bcsr_axpy.argtypes = [VP, ctypes.c_double, VP]
    lib.a2ds_bcsr_apply_bcs.argtypes = [VP]
    lib.a2ds_pc_create.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(VP)]
    lib.a2ds_pc_destroy.argtypes = [VP]
    lib.a2ds_pc_factor.argtypes = [VP, VP]
    lib.a2ds_pc_apply.argtypes = [VP, P_D, P_D]
    lib.a2ds_pc_apply_multi.argtypes = [VP, ctypes.c_int, P_D, P_D]
    lib.a2ds_gmres_solve.argtypes = [VP, VP, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, P_D, P_D, P_I, P_D]
    lib.a2ds_fgmres_solve.argtypes = [VP, VP, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_int, P_D, P_D, P_I]
    lib.a2ds_pc_get.argtypes = [VP, P_I, P_I, P_I, P_I, P_D]
    lib.a2ds_buckling_default_opts.argtypes = [ctypes.POINTER(BucklingOpts)]
    lib.a2ds_buckling_default_opts.restype = None
    lib.a2ds_buckling_solve.argtypes = [VP, ctypes.POINTER(BucklingOpts), P_D, P_D, P_D, P_D, P_D]
    lib.a2ds_buckling_stats.argtypes = [VP, ctypes.c_int, P_D]
    lib.a2ds_eigen_shift_invert.argtypes = [VP, ctypes.POINTER(BucklingOpts), VP, VP, P_D, P_D,
                                            P_D]
    lib.a2ds_eig_sens_thickness.argtypes = [VP, ctypes.c_int, P_D]
    lib.a2ds_newton_preload.argtypes = [VP, P_D, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, P_D, P_I, P_D]
    lib.a2ds_preload_buckling.argtypes = [VP, ctypes.POINTER(BucklingOpts), P_D, P_D, P_D, P_D]
    lib.a2ds_preload_xpt_sens.argtypes = [VP, ctypes.c_int, ctypes.c_double, P_D]
    lib.a2ds_bcsr_time_mult.argtypes = [VP, ctypes.c_int, ctypes.c_int, P_D]
    lib.a2ds_bcsr_time_mult_df.argtypes = [VP, ctypes.c_int, ctypes.c_int, P_D]
    lib.a2ds_eig_sens_xpts.argtypes = [VP, ctypes.c_int, ctypes.c_double, P_D]
    lib.a2ds_add_mat_xpt_sens_inner_product.argtypes = [VP, ctypes.c_int, ctypes.c_double, P_D,
                                                        P_D, P_D, ctypes.c_double, P_D]
    lib.a2ds_add_mat_dv_sens_inner_product.argtypes = [VP, ctypes.c_int, ctypes.c_double, P_D,
                                                       P_D, P_D, P_D]
    lib.a2ds_add_adjoint_res_xpt_sens_product.argtypes = [VP, ctypes.c_double, P_D, P_D,
                                                          ctypes.c_double, P_D]
    lib.a2ds_eval_mat_sv_sens_inner_product.argtypes = [VP, ctypes.c_int, P_D, P_D, P_D,
                                                        ctypes.c_double, P_D]
    lib.a2ds_bdf_scan.argtypes = [ctypes.c_char_p, ctypes.POINTER(VP)]
    lib.a2ds_bdf_destroy.argtypes = [VP]
    lib.a2ds_bdf_get_sizes.argtypes = [VP, P_I, P_I, P_I, P_I, P_I, P_I]
    lib.a2ds_bdf_get_connectivity.argtypes = [VP, P_I, P_I, P_I, P_D]
    lib.a2ds_bdf_get_bcs.argtypes = [VP, P_I, P_I, P_I, P_D]
    lib.a2ds_bdf_get_element_descript.argtypes = [VP, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    lib.a2ds_bdf_get_component_descript.argtypes = [VP, ctypes.c_int, ctypes.c_char_p,
                                                    ctypes.c_int]
    lib.a2ds_write_f5.argtypes = [VP, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_char_p), P_I, P_D, ctypes.c_double]
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        raise A2dsError(rc, _lib.a2ds_last_error().decode())


def _d(a):
    return None if a is None else a.ctypes.data_as(P_D)


def _i(a):
    return None if a is None else a.ctypes.data_as(P_I)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class Assembler:
    """TACSAssembler for one shell element type (Quad4 / Quad9, linear or
    nonlinear strain), one GPU."""

    def __init__(self, X, conn, nonlinear=False):
        self.lib = load()
        X = _f64(X).reshape(-1, 3)
        conn = _i32(conn)
        self.num_nodes, self.num_elements = X.shape[0], conn.shape[0]
        self.nodes_per_elem = conn.shape[1]
        h = VP()
        _check(self.lib.a2ds_mesh_create(self.num_nodes, self.num_elements,
                                         self.nodes_per_elem, _i(conn), _d(X),
                                         int(bool(nonlinear)), ctypes.byref(h)))
        self.h = h
        self._keep = (X, conn)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.a2ds_mesh_destroy(self.h)
            self.h = None

    def set_material(self, E, nu, alpha=0.0, temperature=0.0):
        _check(self.lib.a2ds_mesh_set_material(self.h, E, nu, alpha, temperature))

    def set_yield_stress(self, ys):
        """ys of TACSMaterialProperties (failure values of the .f5 extras)."""
        _check(self.lib.a2ds_mesh_set_yield_stress(self.h, float(ys)))

    def set_thickness(self, t, elem_group=None):
        t = _f64(np.atleast_1d(t))
        g = _i32(elem_group)
        _check(self.lib.a2ds_mesh_set_thickness(self.h, t.size, _d(t), _i(g)))

    def add_bcs(self, nodes, masks, vals=None):
        nodes, masks = _i32(nodes), _i32(masks)
        vals = _f64(vals)
        _check(self.lib.a2ds_mesh_add_bcs(self.h, nodes.size, _i(nodes), _i(masks), _d(vals)))

    def plan(self, order=A2DS_NATURAL_ORDER):
        """Host-only pattern and ordering (no GPU needed)."""
        _check(self.lib.a2ds_mesh_plan(self.h, order))

    def initialize(self, order=A2DS_NATURAL_ORDER):
        _check(self.lib.a2ds_mesh_initialize(self.h, order))

    def get_pattern(self):
        nz = ctypes.c_int()
        _check(self.lib.a2ds_mesh_get_pattern(self.h, ctypes.byref(nz), None, None))
        rowp = np.zeros(self.num_nodes + 1, np.int32)
        cols = np.zeros(nz.value, np.int32)
        _check(self.lib.a2ds_mesh_get_pattern(self.h, None, _i(rowp), _i(cols)))
        return rowp, cols

    def ilu_pattern(self, lev_fill):
        nz = ctypes.c_int()
        _check(self.lib.a2ds_mesh_ilu_pattern(self.h, lev_fill, ctypes.byref(nz), None, None))
        rowp = np.zeros(self.num_nodes + 1, np.int32)
        cols = np.zeros(nz.value, np.int32)
        _check(self.lib.a2ds_mesh_ilu_pattern(self.h, lev_fill, None, _i(rowp), _i(cols)))
        return rowp, cols

    def get_ordering(self):
        p = np.zeros(self.num_nodes, np.int32)
        _check(self.lib.a2ds_mesh_get_ordering(self.h, _i(p)))
        return p

    def node_csr(self, nodiag=False):
        nnz = ctypes.c_int()
        _check(self.lib.a2ds_mesh_node_csr(self.h, int(nodiag), ctypes.byref(nnz), None, None))
        rowp = np.zeros(self.num_nodes + 1, np.int32)
        cols = np.zeros(nnz.value, np.int32)
        _check(self.lib.a2ds_mesh_node_csr(self.h, int(nodiag), None, _i(rowp), _i(cols)))
        return rowp, cols

    def create_mat(self):
        return BCSRMat(self)

    def assemble_mat_type(self, mat_type, A, vars_=None, scatter=A2DS_SCATTER_ATOMIC):
        v = _f64(vars_)
        _check(self.lib.a2ds_assemble_mat_ex(self.h, mat_type, _d(v), A.h, scatter))

    def assemble_res(self, vars_=None):
        v = _f64(vars_)
        res = np.zeros((self.num_nodes, 6))
        _check(self.lib.a2ds_assemble_res(self.h, _d(v), _d(res)))
        return res

    def assemble_jacobian(self, A, vars_=None, want_res=True):
        v = _f64(vars_)
        res = np.zeros((self.num_nodes, 6)) if want_res else None
        _check(self.lib.a2ds_assemble_jacobian(self.h, _d(v), _d(res), A.h))
        return res

    def add_mat_xpt_sens_inner_product(self, scale, mat_type, psi, phi, dfdX=None, vars_=None,
                                       dh=1e-7):
        """dfdX += scale * d(psi^T M phi)/dX (num_nodes x 3), M = K at vars_
        or G along vars_; element-by-element central differences with step
        dh (TACSElement::addMatXptSensInnerProduct)."""
        if dfdX is None:
            dfdX = np.zeros((self.num_nodes, 3))
        assert dfdX.dtype == np.float64 and dfdX.flags.c_contiguous
        ps, ph, v = _f64(psi), _f64(phi), _f64(vars_)
        for a in (ps, ph) + (() if v is None else (v,)):
            if a.size != self.num_nodes * 6:
                raise ValueError("vectors are num_nodes x 6")
        if dfdX.size != self.num_nodes * 3:
            raise ValueError("dfdX is num_nodes x 3")
        _check(self.lib.a2ds_add_mat_xpt_sens_inner_product(
            self.h, int(mat_type), float(scale), _d(ps), _d(ph), _d(v), float(dh), _d(dfdX)))
        return dfdX

    def add_mat_dv_sens_inner_product(self, scale, mat_type, psi, phi, dfdx, vars_=None):
        """dfdx[g] += scale * d(psi^T M phi)/dt_g per thickness group, M = K at
        vars_ or G along vars_ (TACSElement::addMatDVSensInnerProduct, exact
        here)."""
        assert dfdx.dtype == np.float64 and dfdx.flags.c_contiguous
        ps, ph, v = self._vec6(psi), self._vec6(phi), self._vec6(vars_)
        _check(self.lib.a2ds_add_mat_dv_sens_inner_product(
            self.h, int(mat_type), float(scale), _d(ps), _d(ph), _d(v), _d(dfdx)))
        return dfdx

    def _vec6(self, a):
        a = _f64(a)
        if a is not None and a.size != self.num_nodes * 6:
            raise ValueError("vectors are num_nodes x 6")
        return a

    def add_adjoint_res_xpt_sens_products(self, scale, psi, dfdX=None, vars_=None, dh=1e-7):
        """dfdX += scale * psi^T dR(X, vars_)/dX (num_nodes x 3), element by
        element central differences (TACSElement::addAdjResXptProduct)."""
        if dfdX is None:
            dfdX = np.zeros((self.num_nodes, 3))
        if not (dfdX.dtype == np.float64 and dfdX.flags.c_contiguous
                and dfdX.size == self.num_nodes * 3):
            raise ValueError("dfdX is a contiguous float64 num_nodes x 3 array")
        ps, v = self._vec6(psi), self._vec6(vars_)
        _check(self.lib.a2ds_add_adjoint_res_xpt_sens_product(
            self.h, float(scale), _d(ps), _d(v), float(dh), _d(dfdX)))
        return dfdX

    def eval_mat_sv_sens_inner_product(self, mat_type, psi, phi, vars_=None, dh=1e-7):
        """d(psi^T M(vars_) phi)/d(vars_) (num_nodes x 6, Dirichlet entries
        zero), element by element central differences
        (TACSElement::getMatSVSensInnerProduct)."""
        ps, ph, v = self._vec6(psi), self._vec6(phi), self._vec6(vars_)
        out = np.zeros((self.num_nodes, 6))
        _check(self.lib.a2ds_eval_mat_sv_sens_inner_product(
            self.h, int(mat_type), _d(ps), _d(ph), _d(v), float(dh), _d(out)))
        return out


class BCSRMat:
    """Device BCSR matrix in the assembler's ordering."""

    def __init__(self, assembler: Assembler):
        self.a = assembler
        self.lib = assembler.lib
        h = VP()
        _check(self.lib.a2ds_bcsr_create(assembler.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.a2ds_bcsr_destroy(self.h)
            self.h = None

    def sizes(self):
        """(block rows, 6x6 blocks)"""
        nr, nz = ctypes.c_int(), ctypes.c_int()
        _check(self.lib.a2ds_bcsr_get(self.h, ctypes.byref(nr), ctypes.byref(nz), None, None,
                                      None))
        return nr.value, nz.value

    def get_arrays(self):
        nr, nz = ctypes.c_int(), ctypes.c_int()
        _check(self.lib.a2ds_bcsr_get(self.h, ctypes.byref(nr), ctypes.byref(nz), None, None,
                                      None))
        rowp = np.zeros(nr.value + 1, np.int32)
        cols = np.zeros(nz.value, np.int32)
        vals = np.zeros((nz.value, 6, 6))
        _check(self.lib.a2ds_bcsr_get(self.h, None, None, _i(rowp), _i(cols), _d(vals)))
        return rowp, cols, vals

    def set_values(self, vals):
        v = _f64(vals)
        _check(self.lib.a2ds_bcsr_set_values(self.h, _d(v)))

    def mult(self, x):
        x = _f64(x).reshape(-1, 6)
        y = np.zeros_like(x)
        _check(self.lib.a2ds_bcsr_mult(self.h, _d(x), _d(y)))
        return y

    def time_mult(self, nvec=1, iters=20):
        """Device milliseconds per product with nvec device-resident vectors."""
        ms = ctypes.c_double(0.0)
        _check(self.lib.a2ds_bcsr_time_mult(self.h, int(nvec), int(iters), ctypes.byref(ms)))
        return ms.value

    def time_mult_df(self, nvec=4, iters=20):
        """Device milliseconds per double-float product (the matrix as
        double-float pairs) with nvec device-resident FP32 vectors: the
        product of the mixed-precision GMRES-IR inner loop."""
        ms = ctypes.c_double(0.0)
        _check(self.lib.a2ds_bcsr_time_mult_df(self.h, int(nvec), int(iters), ctypes.byref(ms)))
        return ms.value

    def mult_rows(self, x, noalloc=False):
        """y = A x with x, y in the matrix (row) ordering; noalloc=True uses
        the entry point that allocates no device memory (65536 rows at most)."""
        x = _f64(x).reshape(-1, 6)
        y = np.zeros_like(x)
        fn = self.lib.a2ds_bcsr_mult_rows_noalloc if noalloc else self.lib.a2ds_bcsr_mult_rows
        _check(fn(self.h, _d(x), _d(y)))
        return y

    def copy_values(self, other):
        _check(self.lib.a2ds_bcsr_copy(self.h, other.h))

    def axpy(self, alpha, other):
        _check(self.lib.a2ds_bcsr_axpy(self.h, float(alpha), other.h))

    def apply_bcs(self):
        _check(self.lib.a2ds_bcsr_apply_bcs(self.h))

    def to_dense_nodes(self):
        """Dense (6n x 6n) matrix in the caller's node numbering."""
        rowp, cols, vals = self.get_arrays()
        perm = self.a.get_ordering()
        n = rowp.size - 1
        A = np.zeros((6 * n, 6 * n))
        for i in range(n):
            r = perm[i]
            for jp in range(rowp[i], rowp[i + 1]):
                c = perm[cols[jp]]
                A[6 * r:6 * r + 6, 6 * c:6 * c + 6] = vals[jp]
        return A


class SchurPc:
    """TACSSchurPc(mat, levFill, fill) on one GPU: block ILU(levFill)
    (levFill >= num_nodes gives the complete LU), FP64 or FP32 factor."""

    def __init__(self, A: BCSRMat, lev_fill: int, precision: int = 64):
        self.A = A
        self.lib = A.lib
        h = VP()
        _check(self.lib.a2ds_pc_create(A.h, int(lev_fill), int(precision), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.a2ds_pc_destroy(self.h)
            self.h = None

    def factor(self, other: BCSRMat = None):
        _check(self.lib.a2ds_pc_factor(self.h, other.h if other is not None else None))

    def apply_factor(self, x):
        x = _f64(x).reshape(-1, 6)
        y = np.zeros_like(x)
        _check(self.lib.a2ds_pc_apply(self.h, _d(x), _d(y)))
        return y

    def apply_factor_multi(self, X):
        """applyFactor on nrhs stacked vectors X (nrhs, num_nodes, 6)."""
        X = _f64(X)
        Y = np.zeros_like(X)
        _check(self.lib.a2ds_pc_apply_multi(self.h, X.shape[0], _d(X), _d(Y)))
        return Y

    def get_arrays(self):
        nr, nz = ctypes.c_int(), ctypes.c_int()
        _check(self.lib.a2ds_pc_get(self.h, ctypes.byref(nr), ctypes.byref(nz), None, None, None))
        rowp = np.zeros(nr.value + 1, np.int32)
        cols = np.zeros(nz.value, np.int32)
        vals = np.zeros((nz.value, 6, 6))
        _check(self.lib.a2ds_pc_get(self.h, None, None, _i(rowp), _i(cols), _d(vals)))
        return rowp, cols, vals


def gmres_solve(A: "BCSRMat", pc: "SchurPc", b, msub=30, nrestart=15, rtol=1e-12, atol=1e-30,
                raise_on_noconv=True):
    """GMRES(mat, pc, msub, nrestart) solve(b, x) (src/bpmat/KSM.cpp:785):
    returns (x, iterations, residual estimate)."""
    b = _f64(b).reshape(-1, 6)
    x = np.zeros_like(b)
    it, rn = ctypes.c_int(), ctypes.c_double()
    rc = A.lib.a2ds_gmres_solve(A.h, pc.h if pc is not None else None, int(msub), int(nrestart),
                                float(rtol), float(atol), _d(b), _d(x), ctypes.byref(it),
                                ctypes.byref(rn))
    if rc != 6 or raise_on_noconv:
        _check(rc)
    return x, it.value, rn.value


def fgmres_solve(A: "BCSRMat", pc: "SchurPc", b, msub=24, nrestart=8, rtol=1e-10,
                 raise_on_noconv=True):
    """GMRES(mat, pc, msub, nrestart, isFlexible=1) as GMRES-IR: b is one
    (num_nodes, 6) vector or a stack (nrhs, num_nodes, 6) of 1, 2, 4, 8 or 16;
    returns (x, Arnoldi steps).  Convergence is judged on the FP64 residual."""
    b = _f64(b)
    single = b.ndim == 2
    bb = np.ascontiguousarray(b.reshape(-1, A.a.num_nodes, 6) if not single else b[None])
    x = np.zeros_like(bb)
    it = ctypes.c_int()
    rc = A.lib.a2ds_fgmres_solve(A.h, pc.h, int(msub), int(nrestart), float(rtol),
                                 int(bb.shape[0]), _d(bb), _d(x), ctypes.byref(it))
    if rc != 6 or raise_on_noconv:
        _check(rc)
    return (x[0] if single else x), it.value


STAT_NAMES = ["total_s", "assemble_k_s", "assemble_g_s", "factor_s", "path_s", "lanczos_s",
              "lanczos_vectors", "inner_iters", "kernel_launches", "solve_event_ms",
              "factor_a_event_ms", "factor_k_event_ms", "factor_nnzb", "factor_levels",
              "factor_flops", "block_size", "block_iters", "trisolve_ms", "trisolve_calls",
              "gmres_ir_iters", "gmres_ir_cycles"]


class LinearBuckling:
    """TACSLinearBuckling(assembler, sigma, ..., max_lanczos, num_eigvals,
    eig_tol): solve(rhs) then extract_eigenvalue / extract_eigenvector."""

    def __init__(self, assembler: Assembler, sigma, max_lanczos=100, num_eigvals=10,
                 eig_tol=1e-10, lev_fill=1000000, precision=64, seed=0, block_size=4,
                 gmres_m=30, gmres_restarts=15, gmres_rtol=1e-12, gmres_atol=1e-30):
        self.a = assembler
        self.lib = assembler.lib
        o = BucklingOpts()
        self.lib.a2ds_buckling_default_opts(ctypes.byref(o))
        o.sigma, o.max_lanczos, o.num_eigvals, o.eig_tol = sigma, max_lanczos, num_eigvals, eig_tol
        o.lev_fill, o.precision, o.seed, o.block_size = lev_fill, precision, seed, block_size
        o.gmres_m, o.gmres_restarts = gmres_m, gmres_restarts
        o.gmres_rtol, o.gmres_atol = gmres_rtol, gmres_atol
        self.opts = o
        self.eigvals = self.errors = self.eigvecs = self.path = None

    def solve(self, rhs=None, want_vectors=True):
        n, k = self.a.num_nodes, self.opts.num_eigvals
        rhs = _f64(rhs)
        lam, err = np.zeros(k), np.zeros(k)
        vecs = np.zeros((k, n, 6)) if want_vectors else None
        path = np.zeros((n, 6))
        rc = self.lib.a2ds_buckling_solve(self.a.h, ctypes.byref(self.opts), _d(rhs), _d(lam),
                                          _d(err), _d(vecs), _d(path))
        # on A2DS_ERR_NOCONV the current Ritz pairs are still returned
        self.eigvals, self.errors, self.eigvecs, self.path = lam, err, vecs, path
        _check(rc)
        return lam

    def solve_matrices(self, K: "BCSRMat", G: "BCSRMat", want_vectors=True):
        """SEP::solve with EPBucklingShiftInvert(sigma, K, G) on given
        matrices (e.g. K_T(u) and G(u) about a preloaded state)."""
        n, k = self.a.num_nodes, self.opts.num_eigvals
        lam, err = np.zeros(k), np.zeros(k)
        vecs = np.zeros((k, n, 6)) if want_vectors else None
        rc = self.lib.a2ds_eigen_shift_invert(self.a.h, ctypes.byref(self.opts), K.h, G.h,
                                              _d(lam), _d(err), _d(vecs))
        self.eigvals, self.errors, self.eigvecs = lam, err, vecs
        _check(rc)
        return lam

    def solve_preloaded(self, u, want_vectors=True):
        """Buckling about the preloaded state u: K_T(u) x + lam G(u) x = 0
        (a2ds_preload_buckling)."""
        n, k = self.a.num_nodes, self.opts.num_eigvals
        uu = _f64(u)
        lam, err = np.zeros(k), np.zeros(k)
        vecs = np.zeros((k, n, 6)) if want_vectors else None
        rc = self.lib.a2ds_preload_buckling(self.a.h, ctypes.byref(self.opts), _d(uu), _d(lam),
                                            _d(err), _d(vecs))
        self.eigvals, self.errors, self.eigvecs = lam, err, vecs
        _check(rc)
        return lam

    def eval_preload_xpt_sens(self, n, dh=1e-7):
        """dlambda_n/dX about the preloaded state (a2ds_preload_xpt_sens)."""
        out = np.zeros((self.a.num_nodes, 3))
        _check(self.lib.a2ds_preload_xpt_sens(self.a.h, int(n), float(dh), _d(out)))
        return out

    def stats(self):
        out = np.zeros(len(STAT_NAMES))
        _check(self.lib.a2ds_buckling_stats(self.a.h, out.size, _d(out)))
        return dict(zip(STAT_NAMES, out.tolist()))

    def extract_eigenvalue(self, n):
        return self.eigvals[n], self.errors[n]

    def extract_eigenvector(self, n):
        return self.eigvals[n], self.eigvecs[n], self.errors[n]

    def eig_sens_thickness(self, n, num_groups):
        out = np.zeros(num_groups)
        _check(self.lib.a2ds_eig_sens_thickness(self.a.h, int(n), _d(out)))
        return out

    def eval_eigen_xpt_sens(self, n, dh=1e-7):
        """TACSLinearBuckling::evalEigenXptSens: dlambda_n/dX, num_nodes x 3."""
        out = np.zeros((self.a.num_nodes, 3))
        _check(self.lib.a2ds_eig_sens_xpts(self.a.h, int(n), float(dh), _d(out)))
        return out


A2DS_F5_CONNECTIVITY, A2DS_F5_NODES, A2DS_F5_DISPLACEMENTS = 1, 2, 4
A2DS_F5_STRAINS, A2DS_F5_STRESSES, A2DS_F5_EXTRAS, A2DS_F5_LOADS = 8, 16, 32, 64


class ToFH5:
    """TACSToFH5 for shell meshes (src/io/TACSToFH5.h): every output class
    (connectivity, nodes, displacements, strains, stresses, extras, loads)
    written as a .f5 file; loads and the element classes need an
    initialized Assembler, extras its yield stress."""

    def __init__(self, assembler: "Assembler",
                 write_flag=A2DS_F5_CONNECTIVITY | A2DS_F5_NODES | A2DS_F5_DISPLACEMENTS,
                 elem_component=None):
        self.a, self.lib = assembler, assembler.lib
        self.write_flag = write_flag
        self.elem_component = _i32(elem_component)
        ncomp = 1 if elem_component is None else int(np.max(elem_component)) + 1
        self.names = [None] * ncomp

    def set_component_name(self, comp, name):
        if 0 <= comp < len(self.names):
            self.names[comp] = name

    def write_to_file(self, file_name, vars=None, time=0.0):
        vars = _f64(vars)
        arr = (ctypes.c_char_p * len(self.names))(
            *[None if n is None else n.encode() for n in self.names])
        _check(self.lib.a2ds_write_f5(self.a.h, os.fsencode(file_name), self.write_flag,
                                      len(self.names), arr, _i(self.elem_component), _d(vars),
                                      float(time)))


class MeshLoader:
    """TACSMeshLoader (src/io/TACSMeshLoader.h) on one process: scan a
    Nastran BDF file, then read back its connectivity and SPC entries or
    build an Assembler from it (createTACS, TACSMeshLoader.cpp:1133, with
    the one-shell-type-per-mesh restriction of this library)."""

    def __init__(self):
        self.lib = load()
        self.h = None

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.a2ds_bdf_destroy(self.h)
            self.h = None

    def scan_bdf_file(self, file_name):
        if self.h:
            self.lib.a2ds_bdf_destroy(self.h)
            self.h = None
        h = VP()
        _check(self.lib.a2ds_bdf_scan(os.fsencode(file_name), ctypes.byref(h)))
        self.h = h
        sz = [ctypes.c_int() for _ in range(6)]
        _check(self.lib.a2ds_bdf_get_sizes(self.h, *[ctypes.byref(v) for v in sz]))
        (self.num_nodes, self.num_elements, self._conn_size, self.num_bcs, self._bc_size,
         self.num_components) = [v.value for v in sz]

    def get_num_nodes(self):
        return self.num_nodes

    def get_num_elements(self):
        return self.num_elements

    def get_num_components(self):
        return self.num_components

    def get_connectivity(self):
        """(elem_node_ptr, elem_node_conn, elem_component, Xpts)"""
        ptr = np.zeros(self.num_elements + 1, np.int32)
        conn = np.zeros(self._conn_size, np.int32)
        comp = np.zeros(self.num_elements, np.int32)
        X = np.zeros((self.num_nodes, 3))
        _check(self.lib.a2ds_bdf_get_connectivity(self.h, _i(ptr), _i(conn), _i(comp), _d(X)))
        return ptr, conn, comp, X

    def get_bcs(self):
        """(bc_nodes, bc_vars, bc_ptr, bc_vals)"""
        nodes = np.zeros(self.num_bcs, np.int32)
        ptr = np.zeros(self.num_bcs + 1, np.int32)
        var = np.zeros(self._bc_size, np.int32)
        vals = np.zeros(self._bc_size)
        _check(self.lib.a2ds_bdf_get_bcs(self.h, _i(nodes), _i(var), _i(ptr), _d(vals)))
        return nodes, var, ptr, vals

    def get_element_descript(self, comp):
        buf = ctypes.create_string_buffer(16)
        _check(self.lib.a2ds_bdf_get_element_descript(self.h, comp, buf, 16))
        return buf.value.decode()

    def get_component_descript(self, comp):
        buf = ctypes.create_string_buffer(40)
        _check(self.lib.a2ds_bdf_get_component_descript(self.h, comp, buf, 40))
        return buf.value.decode()

    def bc_masks(self):
        """The SPC entries as add_bcs arrays (nodes, 6-bit masks, num x 6
        values); variables beyond the six shell DOFs are dropped."""
        nodes, var, ptr, vals = self.get_bcs()
        masks = np.zeros(self.num_bcs, np.int32)
        v6 = np.zeros((self.num_bcs, 6))
        for b in range(self.num_bcs):
            for q in range(ptr[b], ptr[b + 1]):
                if var[q] < 6:
                    masks[b] |= 1 << int(var[q])
                    v6[b, var[q]] = vals[q]
        return nodes, masks, v6

    def create_assembler(self, nonlinear=False):
        """An Assembler on the scanned mesh with its SPC entries added; every
        element must be CQUAD4/CQUADR (Quad4 shell) or every element
        CQUAD9/CQUAD (Quad9 shell).  Material, thickness (per component:
        set_thickness(t, elem_group=elem_component)) and initialize() are
        left to the caller."""
        ptr, conn, comp, X = self.get_connectivity()
        npe = np.diff(ptr)
        if self.num_elements == 0 or not (np.all(npe == 4) or np.all(npe == 9)):
            raise A2dsError(-1, "the shell assembler needs all Quad4 or all Quad9 elements")
        types = {self.get_element_descript(c) for c in np.unique(comp)}
        allowed = {"CQUAD4", "CQUADR"} if npe[0] == 4 else {"CQUAD9", "CQUAD"}
        if not types <= allowed:
            raise A2dsError(-1, f"element types {sorted(types)} are not shell quads")
        a = Assembler(X, conn.reshape(-1, int(npe[0])), nonlinear=nonlinear)
        nodes, masks, v6 = self.bc_masks()
        if nodes.size:
            a.add_bcs(nodes, masks, v6)
        self.elem_component = comp
        return a
