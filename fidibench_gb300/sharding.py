"""Work split across ranks (one process per GPU).

The plain form does not shard (one field per GPU; ranks run replicas).  A
batch of independent instances shards by instance: a greedy size-balanced
partition (largest first onto the least-loaded rank) with no data exchange
during the advect; afterwards only per-instance results (checksums, gradient
sums) are gathered, and timings are reduced with a max.  torch.distributed
is used only for these host-side collectives (gloo on CPU, nccl on GPU).
"""
from __future__ import annotations

from datetime import timedelta

import numpy as np


def partition_instances(sizes, world_size: int) -> list[list[int]]:
    """Indices of the instances each rank owns, balancing total cells.
    Deterministic: ties broken by instance index, then by rank."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * world_size
    parts: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += int(sizes[i])
    return [sorted(p) for p in parts]


def imbalance(sizes, parts) -> float:
    """max rank load / mean rank load (1.0 = perfect)."""
    loads = [sum(int(sizes[i]) for i in p) for p in parts]
    mean = sum(loads) / max(len(loads), 1)
    return max(loads) / mean if mean else 1.0


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def gather_by_index(local: dict, count: int, fill=np.nan) -> np.ndarray:
    """Every rank passes {instance index: value}; all ranks get the values of
    all `count` instances in index order."""
    dist = _dist()
    out = np.full(count, fill, dtype=np.float64)
    if dist is None:
        for k, v in local.items():
            out[k] = v
        return out
    pieces = [None] * dist.get_world_size()
    dist.all_gather_object(pieces, {int(k): float(v) for k, v in local.items()})
    for p in pieces:
        for k, v in p.items():
            out[k] = v
    return out


def reduce_max(value: float) -> float:
    """Max of a host scalar over ranks (the slowest rank's time)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def init_host_group(rank: int, world_size: int, addr: str, port: int, timeout_s: float = 30.0):
    """A gloo process group for host-side collectives (tests, CPU-only runs)."""
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://{addr}:{port}", rank=rank,
                            world_size=world_size, timeout=timedelta(seconds=timeout_s))
    return dist


__all__ = ["partition_instances", "imbalance", "gather_by_index", "reduce_max",
           "init_host_group"]
