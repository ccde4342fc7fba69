"""The multi-threaded CPU solve (oracle/c/cpu_parallel.c and
oracle.cpu_buckling_solve), the timed CPU baseline and the reference arm of
bench.py: its factorization equals the serial restatement of BCSRMatFactor6
bit for bit, its solves invert the factor, its pattern is a complete
elimination pattern, and its buckling loads of the reference's 32 x 64
cylinder match the fixture's sparse truth (1e-8).  The reference arm loads
no part of the GPU library."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, REPO
from a2ds import mesh as meshgen


@pytest.fixture(scope="module")
def plan16():
    m = meshgen.cylinder(16, 32)
    return m, oracle.CpuPlan(m)


def test_nd_order_is_a_permutation(plan16):
    m, plan = plan16
    assert np.array_equal(np.sort(plan.perm), np.arange(m.num_nodes))


def test_symbolic_pattern_is_closed_under_elimination(plan16):
    m, plan = plan16
    fr, fc, fd = plan.frowp, plan.fcols, plan.fdiag
    n = plan.n
    rows = [set(fc[fr[i]:fr[i + 1]].tolist()) for i in range(n)]
    for i in range(n):
        assert set(plan.cols[plan.rowp[i]:plan.rowp[i + 1]].tolist()) <= rows[i]
        assert np.all(np.diff(fc[fr[i]:fr[i + 1]]) > 0) and fc[fd[i]] == i
        for j in fc[fr[i]:fd[i]]:
            # eliminating pivot j from row i fills U_j's columns into row i
            assert {c for c in fc[fd[j] + 1:fr[j + 1]] if c > j} <= rows[i]


def test_parallel_factor_equals_serial_and_solves(plan16):
    m, plan = plan16
    K = plan.assemble(m, oracle.STIFFNESS)
    F = plan.factor(K)
    F_serial = oracle.factor(plan.rowp, plan.cols, K, plan.frowp, plan.fcols, plan.fdiag)
    assert np.array_equal(F, F_serial)
    x = np.random.default_rng(1).standard_normal((6 * plan.n, 4))
    y = plan.apply(F, x)
    for c in range(4):
        y1 = np.zeros(6 * plan.n)
        lib = oracle.load()
        lib.orc_apply_factor(plan.n, oracle._pi(plan.frowp), oracle._pi(plan.fcols),
                             oracle._pi(plan.fdiag), oracle._p(F),
                             oracle._p(np.ascontiguousarray(x[:, c])), oracle._p(y1))
        assert np.abs(y[:, c] - y1).max() <= 1e-12 * np.abs(y1).max()
    r = plan.spmm(K, y, x)
    assert np.linalg.norm(r) < 1e-5 * np.linalg.norm(x)


def test_cpu_buckling_solve_config1_against_fixture():
    f = np.load(os.path.join(GOLDEN, "cyl_q4_32x64_lu.npz"))
    m = meshgen.cylinder(32, 64)
    assert np.array_equal(m.X, f["X"]) and np.array_equal(m.rhs, f["rhs"])
    plan = oracle.CpuPlan(m)
    lam, t, nvec = oracle.cpu_buckling_solve(m, plan, float(f["sigma"]), neig=10, block=4,
                                             eig_tol=1e-10)
    truth = f["eigvals_sparse"][:10]
    assert np.max(np.abs(lam - truth) / truth) < 1e-8, (lam, truth)


def test_reference_arm_loads_no_gpu_library():
    code = (
        "import sys, json, io, contextlib; sys.argv=['bench.py','--impl','reference','--nx','8',"
        "'--ny','16','--neig','4']; sys.path.insert(0, %r); import bench; buf = io.StringIO()\n"
        "with contextlib.redirect_stdout(buf): rc = bench.main()\n"
        "maps = open('/proc/self/maps').read(); line = json.loads(buf.getvalue())\n"
        "assert rc == 0 and line['impl'] == 'reference' and line['value'] > 0, line\n"
        "assert 'liba2ds_gpu' not in maps\nprint('ok', line['cpu_baseline']['cores'])" % REPO)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, RANK="0", WORLD_SIZE="1"))
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("ok")
