"""Replica-parallel runs: one independent eigenproblem per rank.

Instances (k-points, disorder seeds, requests) are independent, so several GPUs
run replicas with no collective on the data path. The only exchange is the final
throughput aggregation: the whole job's converged modes over the slowest rank's
time.
"""
from __future__ import annotations

import torch


def replica_seed(base_seed: int, rank: int) -> int:
    """Structure and start-vector seed of rank `rank` (rank 0 reproduces the 1-GPU run)."""
    return int(base_seed) + int(rank)


def aggregate(total_s: float, modes: int, device=None) -> tuple[float, float]:
    """(max over ranks of the timed seconds, sum over ranks of converged modes).

    Works on any initialised process group (NCCL on the GPU machine, gloo in tests);
    without one it returns the local values.
    """
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(total_s), float(modes)
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([float(total_s)], dtype=torch.float64, device=dev)
    m = torch.tensor([float(modes)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(m, op=dist.ReduceOp.SUM)
    return float(t[0]), float(m[0])
