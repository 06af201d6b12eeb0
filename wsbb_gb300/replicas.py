"""Host logic of the multi-GPU form: independent replicas, one process per
GPU, no collective on the data path.

The search shards by instance (or by subtree): every rank runs its own
searches and the ranks meet only between runs, to aggregate throughput
(bounded nodes summed, time = the slowest rank) and to exchange
incumbents, the one value a shared search would need (a min over ranks
of the int32 makespan, with the winning rank's permutation broadcast).
Works on any torch.distributed backend: gloo on CPU, NCCL on GPUs.
"""
from __future__ import annotations

import numpy as np


def replica_seed(rank: int, base: int = 0) -> int:
    """Instance seed of a rank under weak scaling: one instance per rank."""
    return base + rank


def _device(group=None):
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def aggregate(bounded: int, seconds: float, group=None) -> tuple[float, float, float]:
    """(total bounded nodes, slowest rank's seconds, whole-job nodes/s)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(bounded), float(seconds), bounded / max(seconds, 1e-12)
    dev = _device(group)
    t = torch.tensor([float(bounded)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(s, op=dist.ReduceOp.MAX, group=group)
    total, slow = float(t.item()), float(s.item())
    return total, slow, total / max(slow, 1e-12)


def min_incumbent(cost: int, perm, group=None) -> tuple[int, np.ndarray, int]:
    """Best incumbent over ranks: (cost, permutation, owning rank); ties go
    to the lowest rank, so every rank gets the same answer."""
    import torch
    import torch.distributed as dist
    perm = np.asarray(perm, dtype=np.int32)
    if not dist.is_available() or not dist.is_initialized():
        return int(cost), perm.copy(), 0
    dev = _device(group)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    # one int64 key: cost first, then rank, so the min is unique
    key = torch.tensor([int(cost) * world + rank], dtype=torch.int64, device=dev)
    dist.all_reduce(key, op=dist.ReduceOp.MIN, group=group)
    k = int(key.item())
    best_cost, owner = k // world, k % world
    buf = torch.from_numpy(perm.astype(np.int64)).to(dev)
    dist.broadcast(buf, src=owner, group=group)
    return best_cost, buf.cpu().numpy().astype(np.int32), owner
