"""Host-side logic of bench.py's multi-process launch on CPU: two gloo ranks
(the GPU run uses one rank per GPU over NCCL with the same code path).

* every rank gets the slowest rank's time from max_over_ranks;
* the reference arm runs on rank 0 only; other ranks return at once.
"""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(10.0 * (rank + 1))
        r, w, lr = bench.dist_env()

        class Args:
            sizes, side, steps, warmup = "1M", 64, 1, 0

        ref = bench.run_reference(Args()) if rank != 0 else "skipped"
        q.put((rank, got, (r, w, lr), ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_rank0_reports():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r: (got, env, ref) for r, got, env, ref in out}
    assert by_rank[0][0] == by_rank[1][0] == 20.0
    assert by_rank[1][1] == (1, 2, 1)
    assert by_rank[1][2] is None  # the reference arm does no work off rank 0


def test_max_over_ranks_without_a_group():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
