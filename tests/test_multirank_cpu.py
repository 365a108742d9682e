"""The multi-GPU path, run on CPU with two gloo ranks.

bench.py --gpus N runs one process per GPU under torch.distributed.run.
Halos and trees are independent, so the path is replicas: each rank evolves
its own batch (seed 2 + rank) and its own forest (seed 3 + rank) with no
collective on the data path, the job's time is the slowest rank's and its
work the sum over ranks (weak scaling).  The reference arm runs on rank 0
only; the other ranks exit at once.  GPU kernels never wait on another rank,
so this host logic is what there is to test with more than one process."""

import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_replicas(tmp_path):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}",
           os.path.join(ROOT, "tests", "multirank_worker.py"), str(tmp_path)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    seen = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(2)]
    for k, s in enumerate(seen):
        assert s["rank"] == k and s["world"] == 2
        # The slowest rank's time and the sum of the ranks' work.
        assert s["elapsed"] == pytest.approx(2.5)
        assert s["work"] == 30
    # Every rank holds the same view of both ranks' inputs, and the inputs
    # differ between ranks (each rank works on its own halos and trees).
    a, b = (np.array(s["checksums"]) for s in seen)
    np.testing.assert_array_equal(a, b)
    assert not np.any(a[0, :3] == a[1, :3])


def test_reduce_without_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, None, 1.25, 7) == (1.25, 7)
    assert bench.reduce_over_ranks(None, None, 1.25) == (1.25, None)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=120, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
