"""The multi-rank paths of bench.py, on CPU with the gloo backend (world size 2).

Replicas only: every rank runs the whole grid, the job's time is the slowest rank's and its
throughput counts every replica's cells (weak scaling).  The reference arm runs on rank 0
alone; the other ranks return without work.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        ms = bench.max_over_ranks(local_ms, world, "cpu")
        value = bench.job_throughput(615888, 6, world, ms)
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, ms, value in got:
        assert ms == 150.0  # every rank sees the slowest rank's time
        assert value == pytest.approx(615888 * 6 * 2 / 0.150)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.5, 1, "cpu") == 42.5
    assert bench.job_throughput(1000, 4, 1, 2000.0) == pytest.approx(2000.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup = 1, 0
    bench.run_reference(Args())  # returns before building or running anything
    assert capsys.readouterr().out == ""
