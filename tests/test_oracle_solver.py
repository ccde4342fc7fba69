"""The CPU oracle's assembly, factorization, solves and buckling solve
against the reference's own outputs (tests/golden/cyl_*.npz and the
stiffened panel, tests/golden/panel_q9_4x8x1_lu.npz)."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from a2ds import mesh as meshgen


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def fixture_mesh(f):
    return meshgen.ShellMesh(X=f["X"], conn=f["conn"], bc_nodes=f["bc_nodes"],
                             bc_mask=f["bc_mask"], bc_vals=f["bc_vals"], rhs=f["rhs"],
                             thickness=f["thickness"],
                             dv_group=np.zeros(f["conn"].shape[0], np.int32),
                             E=float(f["E"]), nu=float(f["nu"]),
                             order=3 if f["conn"].shape[1] == 9 else 2)


def diag_of(rowp, cols):
    return np.array([rowp[i] + np.searchsorted(cols[rowp[i]:rowp[i + 1]], i)
                     for i in range(rowp.size - 1)], np.int32)


def bc_rows(f, perm):
    iperm = np.empty_like(perm)
    iperm[perm] = np.arange(perm.size)
    return iperm[f["bc_nodes"]].astype(np.int32), f["bc_mask"].astype(np.int32)


@pytest.mark.parametrize("case", ["cyl_q4_4x8_lu", "cyl_q4_8x16_ilu1", "cyl_q9_2x4_lu",
                                  "panel_q9_4x8x1_lu"])
def test_oracle_assembly_and_factor(case):
    f = np.load(os.path.join(GOLDEN, case + ".npz"))
    m = fixture_mesh(f)
    perm = f["amd_perm"].astype(np.int32)
    br, bm = bc_rows(f, perm)
    K = oracle.assemble(m, oracle.STIFFNESS, perm, f["bcsr_rowp"], f["bcsr_cols"], None, False,
                        br, bm)
    assert rel(K, f["K_after"]) < 1e-12
    G = oracle.assemble(m, oracle.GEOMETRIC, perm, f["bcsr_rowp"], f["bcsr_cols"], f["path"],
                        False, br, bm)
    assert rel(G, f["G"]) < 1e-11
    fr, fc = f["ilu_rowp"], f["ilu_cols"]
    F = oracle.factor(f["bcsr_rowp"], f["bcsr_cols"], K, fr, fc, diag_of(fr, fc))
    assert rel(F, f["ilu_K"]) < 1e-10


@pytest.mark.parametrize("case", ["cyl_q4_4x8_lu", "cyl_q9_2x4_lu"])
def test_oracle_buckling_matches_reference(case):
    """Same algorithm as the reference (LU of K, GMRES on K + sigma G, 50
    Lanczos steps): the lowest loads agree with the reference's SEP output."""
    f = np.load(os.path.join(GOLDEN, case + ".npz"))
    m = fixture_mesh(f)
    perm = f["amd_perm"].astype(np.int32)
    br, bm = bc_rows(f, perm)
    fr, fc = f["ilu_rowp"], f["ilu_cols"]
    cb = oracle.CpuBuckling(m, perm, f["bcsr_rowp"], f["bcsr_cols"], fr, fc, diag_of(fr, fc),
                            br, bm)
    lam = cb.solve(float(f["sigma"]), f["rhs"], lanczos_iters=int(f["neig"]), num_eig=5,
                   gm_m=int(f["gm_m"]), gm_restarts=int(f["gm_restarts"]))
    assert rel(cb.path, f["path"]) < 1e-9
    ref = f["eigvals"][:5]
    assert np.max(np.abs(lam - ref) / np.abs(ref)) < 1e-8, (lam, ref)


def test_oracle_buckling_panel_lowest_load():
    """The stiffened panel (Quad9 skin and webs): the reference ran 10
    Lanczos steps (num_eigvals = 10, F3), which converge only the lowest
    load; the oracle's path and lowest load agree with the reference's."""
    f = np.load(os.path.join(GOLDEN, "panel_q9_4x8x1_lu.npz"))
    m = fixture_mesh(f)
    perm = f["amd_perm"].astype(np.int32)
    br, bm = bc_rows(f, perm)
    fr, fc = f["ilu_rowp"], f["ilu_cols"]
    cb = oracle.CpuBuckling(m, perm, f["bcsr_rowp"], f["bcsr_cols"], fr, fc, diag_of(fr, fc),
                            br, bm)
    lam = cb.solve(float(f["sigma"]), f["rhs"], lanczos_iters=int(f["neig"]), num_eig=5,
                   gm_m=int(f["gm_m"]), gm_restarts=int(f["gm_restarts"]))
    assert rel(cb.path, f["path"]) < 1e-9
    assert abs(lam[0] - f["eigvals"][0]) < 1e-8 * abs(f["eigvals"][0])
    assert abs(lam[0] - f["eigvals_dense"][0]) < 1e-8 * abs(f["eigvals_dense"][0])
