"""The multi-rank path of bench.py on CPU: two gloo ranks (no GPU) run the
bench's barrier and max-over-ranks, and the whole-job throughput divides the
units of all ranks by the slowest rank's time.  Under torchrun the reference
arm runs on rank 0 only; other ranks exit 0 without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = bench.RankGroup(world, "cpu")
        g.barrier()
        ms = 100.0 + 50.0 * rank  # rank 1 is the slower one
        worst = g.max(ms)
        out[rank] = (worst, bench.aggregate_rate(world, 1000, 10, worst))
        g.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    # 2 ranks x 1000 units x 10 steps over the slowest rank's 150 ms
    assert res[0][1] == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_rank_group_is_local():
    g = bench.RankGroup(1, "cpu")
    g.barrier()
    assert g.max(3.5) == 3.5
    assert bench.aggregate_rate(1, 5.12e6, 10, 1000.0) == pytest.approx(5.12e7)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        nx, nz, degree, cfl, steps, warmup = 320, 160, 4, 5.0, 10, 3

    # rank 1 returns at once: no oracle build, no work
    assert bench.run_reference(Args()) == 0
