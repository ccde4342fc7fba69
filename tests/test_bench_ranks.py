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
