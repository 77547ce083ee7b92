"""Multi-GPU runs are independent replicas: bench.py's barrier and max-over-ranks timing
with two gloo ranks on CPU (no GPU, no collective on the data path)."""

from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench

    r, w = bench.dist_setup()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    ms = bench.reduce_max(10.0 + 5.0 * rank, w)  # each replica's own timed-region length
    out[rank] = ms
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == 15.0


def test_single_process_needs_no_process_group():
    import bench

    assert bench.reduce_max(3.5, 1) == 3.5
    bench.barrier(1)
