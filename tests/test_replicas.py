"""Multi-GPU in this library is replicas only (one dependency DAG per solve does
not shard): bench.py runs one independent solve per rank, takes the slowest
rank's time and reports the whole-job rate.  That host logic is checked here
with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "measured" (1 + r) ms for the step and 0.5 + 2r ms for the kernel
        got = bench.max_over_ranks([1.0 + rank, 0.5 + 2.0 * rank], torch.device("cpu"))
        w, r, _ = bench.dist_env()
        out.put((rank, got, w, r))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, w, r in res:
        assert got == [2.0, 2.5]
        assert (w, r) == (world, rank)


def test_replica_value_is_whole_job_rate():
    flops = 2.0 * 20_966_810 - 4_194_304
    one = bench.replica_value(1, flops, 0.8)
    assert bench.replica_value(4, flops, 0.8) == pytest.approx(4 * one)
    assert one == pytest.approx(flops / 0.8e-3 / 1e9)
