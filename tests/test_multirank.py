"""The N > 1 path of bench.py on CPU: two gloo ranks (world size 2).

The benchmark runs one replica per GPU with no data-path collective; the job's
time is the slowest rank's (an all-reduce MAX) and its throughput counts the
units of every rank.  Under torchrun the reference arm runs on rank 0 alone and
the other ranks exit 0 without work.
"""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [7.0, 11.0][rank]  # the second rank is the slower one
        ms = bench.max_over_ranks(local_ms, world, device="cpu")
        value = bench.job_throughput(1000, world, ms * 1e-3)
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_count_all_units():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    assert set(out.keys()) == {0, 1}
    for rank in (0, 1):
        ms, value = out[rank]
        assert ms == 11.0
        assert value == pytest.approx(2 * 1000 / 11e-3)


def test_single_rank_needs_no_collective():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(10, 1, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
