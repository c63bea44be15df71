"""Replica execution of batched skew solves over several processes, one GPU each.

Batched work shards by matrix: every matrix is independent, so each process
(rank) builds a ``BatchPlan`` over its own shard and runs it on its own GPU with
no collective on the data path.  The only exchanges are on the host side and
outside the timed solve: the per-matrix scalars (log|Pf|, sign, status) gathered
back into the caller's order, and the max-over-ranks of a step time.  A single
large matrix does not shard (the blocked reduction of one matrix stays on one
GPU), so it runs as independent replicas.

The process group may use any backend; tensors passed to the collectives live
on ``device`` (``cuda`` for NCCL, ``cpu`` for gloo).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np


def matrix_cost(sizes: Sequence[int]) -> np.ndarray:
    """Work per matrix used for balancing: the n^3 of the Householder reduction."""
    n = np.asarray(sizes, dtype=np.float64)
    return n ** 3


def shard_indices(sizes: Sequence[int], world: int, rank: int) -> np.ndarray:
    """Indices of the matrices that ``rank`` solves, balanced by n^3.

    Longest-processing-time greedy: matrices in decreasing cost (ties by index)
    go to the currently least loaded rank (ties by rank).  Deterministic, so all
    ranks compute the same partition without communicating.  Each shard is
    returned in increasing index order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of world {world}")
    cost = matrix_cost(sizes)
    order = sorted(range(len(cost)), key=lambda i: (-cost[i], i))
    load = np.zeros(world)
    owner = np.empty(len(cost), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))  # first minimum: lowest rank on ties
        owner[i] = r
        load[r] += cost[i]
    return np.nonzero(owner == rank)[0].astype(np.int64)


def gather_scalars(local_idx: np.ndarray, local_values: np.ndarray, count: int, dist=None,
                   device: str = "cpu") -> np.ndarray:
    """All ranks' per-matrix scalars, back in the global order (every rank gets all).

    ``local_values`` is float64 (cast from int status as needed) aligned with
    ``local_idx``.  Without a process group the local values are scattered
    into a full array directly."""
    out = np.full(count, np.nan)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        out[np.asarray(local_idx, dtype=np.int64)] = local_values
        return out
    import torch

    world = dist.get_world_size()
    m = torch.tensor([len(local_idx)], dtype=torch.int64, device=device)
    counts = [torch.zeros(1, dtype=torch.int64, device=device) for _ in range(world)]
    dist.all_gather(counts, m)
    cap = int(max(int(c.item()) for c in counts))
    pad_i = torch.full((cap,), -1, dtype=torch.int64, device=device)
    pad_v = torch.zeros(cap, dtype=torch.float64, device=device)
    if len(local_idx):
        pad_i[: len(local_idx)] = torch.as_tensor(np.asarray(local_idx, dtype=np.int64), device=device)
        pad_v[: len(local_idx)] = torch.as_tensor(np.asarray(local_values, dtype=np.float64), device=device)
    all_i = [torch.empty_like(pad_i) for _ in range(world)]
    all_v = [torch.empty_like(pad_v) for _ in range(world)]
    dist.all_gather(all_i, pad_i)
    dist.all_gather(all_v, pad_v)
    for ti, tv in zip(all_i, all_v):
        i = ti.cpu().numpy()
        v = tv.cpu().numpy()
        keep = i >= 0
        out[i[keep]] = v[keep]
    return out


def max_over_ranks(x: float, dist=None, device: str = "cpu") -> float:
    """The maximum of a per-rank scalar (e.g. a step time) over all ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_scaling_throughput(units_per_rank: int, world: int, steps: int, seconds: float) -> float:
    """Whole-job throughput when every rank processes ``units_per_rank`` per step:
    all ranks' units over the slowest rank's time."""
    if seconds <= 0:
        raise ValueError("non-positive time")
    return world * units_per_rank * steps / seconds


def init_from_env(backend: str, device_id: Optional[int] = None):
    """(world, rank, local_rank, dist or None) from the torchrun environment;
    initialises the default process group when WORLD_SIZE > 1."""
    import os

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return 1, 0, local, None
    import torch
    import torch.distributed as dist

    if backend == "nccl":
        dist.init_process_group("nccl", device_id=torch.device("cuda", local if device_id is None else device_id))
    else:
        dist.init_process_group(backend)
    return world, rank, local, dist
