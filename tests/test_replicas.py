"""The multi-GPU form of this path is replicas: frequencies are independent,
so each rank runs the whole workload on its own GPU with no collective in the
data path, and the job reports the slowest rank's step time.  The host-side
rank logic of bench.py runs here on CPU with two gloo ranks."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        import bench

        ms = bench.max_over_ranks(times[rank], dist, "cpu")
        value = bench.job_value(2.706e11, world, ms)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fp:
            json.dump({"ms": ms, "value": value}, fp)
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    times = [0.9, 1.2]  # ms per step on each rank
    mp.spawn(_rank, args=(2, _free_port(), times, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        with open(tmp_path / f"rank{rank}.json") as fp:
            r = json.load(fp)
        assert r["ms"] == pytest.approx(1.2)  # every rank sees the job's time
        # whole-job throughput: both ranks' work over the slowest rank's time
        assert r["value"] == pytest.approx(2 * 2.706e11 / 1.2e-3)
    assert torch.distributed.is_available()


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(0.75, None, "cpu") == pytest.approx(0.75)
    assert bench.job_value(1e9, 1, 0.5) == pytest.approx(2e12)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank starts bench.py --impl reference; rank 0
    alone times the CPU reference and prints, the others exit 0 at once."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
