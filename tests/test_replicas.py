"""Replica-parallel aggregation over a 2-rank gloo process group on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    import torch.distributed as dist
    from eigenfns_gb300.replicas import aggregate, replica_seed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r times (2 + r) seconds and converges (100 + 10 r) modes
        total, modes = aggregate(2.0 + rank, 100 + 10 * rank)
        q.put((rank, total, modes, replica_seed(7, rank)))
    finally:
        dist.destroy_process_group()


def test_aggregate_takes_slowest_rank_and_sums_modes():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, total, modes, seed in got:
        assert total == 3.0 and modes == 210.0     # max time, summed modes
        assert seed == 7 + rank                    # distinct replica per rank
    assert got[0][3] == 7                          # rank 0 reproduces the 1-GPU run


def test_aggregate_without_process_group_is_local():
    from eigenfns_gb300.replicas import aggregate
    assert aggregate(1.5, 12) == (1.5, 12.0)
