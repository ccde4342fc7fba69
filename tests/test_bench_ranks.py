"""bench.py's multi-GPU host logic on CPU: replicas, one per rank, timed
independently; the whole-job timing is each figure's maximum over the
ranks (gloo, world size 2), and the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

CHILD = r"""
import os, sys
sys.path.insert(0, os.environ["REPO"])
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"])
dist.init_process_group("gloo")
got = bench.max_over_ranks([1.0 + rank, 5.0 - rank], dist)
assert got == [2.0, 5.0], got
assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
dist.barrier()
dist.destroy_process_group()
print("ok", rank)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_gloo_world_2():
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, REPO=REPO, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for rank, p in enumerate(procs):
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        assert f"ok {rank}" in out


def test_reference_arm_other_ranks_do_no_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_loads_fixture_is_the_bench_workload():
    """The 512x1024 reference-loads fixture (the GPU test's truth at the bench
    size) was made on the benchmark's own workload: the same mesh size and
    the same shift bench.py uses, and its loads lie above that shift."""
    import numpy as np

    sys.path.insert(0, REPO)
    import bench
    f = np.load(os.path.join(REPO, "tests", "golden", "cyl_q4_512x1024_ref_loads.npz"))
    m = bench.build_workload(int(f["nx"]), int(f["ny"]))
    assert (int(f["nx"]), int(f["ny"])) == (512, 1024)
    assert float(f["sigma"]) == pytest.approx(bench.workload_sigma(m), rel=1e-15)
    lam = np.asarray(f["eigvals"])
    assert lam.size == 10 and np.all(np.diff(lam) >= 0) and lam[0] > float(f["sigma"])
