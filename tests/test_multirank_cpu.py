"""The multi-GPU path, run on CPU with two gloo ranks.

bench.py --gpus N runs one process per GPU under torch.distributed.run with
no collective on the data path (weak scaling): each rank evolves its own
isolated halos (seed 2 + rank), and one forest is split over the ranks
by longest processing time first on node counts (the reference hands out
forests largest first, tasks/evolve_forests/work_share/_class.F90:37); the
job's time is the slowest rank's and its work the sum over ranks.  The
reference arm runs on rank 0 only; the other ranks exit at once.  GPU
kernels never wait on another rank, so the split and the gathering are
what there is to test with more than one process: each rank evolves its
share of the forest with the CPU oracle, and the union of the shares must
be the whole forest evolved by one process, bit for bit."""

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


def test_two_gloo_ranks(tmp_path):
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
    # Every rank holds the same view of both ranks' halos, and the halos
    # differ between ranks.
    a, b = (np.array(s["checksums"]) for s in seen)
    np.testing.assert_array_equal(a, b)
    assert not np.any(a[0] == a[1])
    # The forest: every tree on exactly one rank, the loads balanced to
    # within the largest tree, and the union of the ranks' results equal to
    # the one-process evolution bit for bit.
    split = json.load(open(tmp_path / "split.json"))
    trees = sorted(split["trees"][0] + split["trees"][1])
    assert trees == list(range(len(split["tree_nodes"])))
    assert abs(split["nodes"][0] - split["nodes"][1]) <= max(split["tree_nodes"])
    assert [r[1] for r in split["per_rank"]] == split["nodes"]
    union, single = np.load(tmp_path / "union.npy"), np.load(tmp_path / "single.npy")
    assert not np.isnan(union).any()
    np.testing.assert_array_equal(union, single)


def test_lpt_assignment():
    """Largest tree first, each to the least-loaded rank."""
    sys.path.insert(0, ROOT)
    from galacticus_gb300 import forest
    sizes = [5, 1, 9, 3, 3, 7]
    tree = np.repeat(np.arange(len(sizes)), sizes).astype(np.int32)
    f = forest.Forest(tree, *[np.zeros(len(tree), np.int32)] * 3, *[np.zeros(len(tree))] * 3)
    a = forest.lpt_assignment(f, 2)
    # 9 -> r0; 7 -> r1; 5 -> r1 (7 < 9); 3 -> r0 (9 < 12); 3 -> r0 (12 = 12:
    # the lower rank); 1 -> r1 (12 < 15).
    assert a[0].tolist() == [2, 3, 4] and a[1].tolist() == [0, 1, 5]
    assert forest.lpt_assignment(f, 1)[0].tolist() == list(range(len(sizes)))


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
