"""Work over several GPUs: one process per GPU, no collective on the data
path, one all-reduce of n_q doubles at the end.

* Ensembles: members sharded across ranks (below).
* One structure: ``Debye.calc_shard(bodies, rank, world)`` computes a
  contiguous run of the forward work items (balanced by pair count) and
  returns its additive FP64 contribution to I(q); ``combine_shards`` sums
  the contributions over ranks.

Members of an ensemble are independent structures, so each rank runs its own
share through one ``DebyeBatch`` (one graph-captured persistent pass) and the
ranks meet only once, to combine the per-rank curve sums into the ensemble
average (n_q doubles per rank).  The reference runs an ensemble as a loop of
``calc`` calls over the models on one device (calc_saxs/calc_saxs.hpp:611-624,
``avg_ensemble``); the average is the same, the sum is split.

    parts = partition_members(sizes, world)           # same on every rank
    mine = parts[rank]
    with DebyeBatch(q, ff, [sizes[m] for m in mine], device=local) as b:
        curves = b.forward([members[m] for m in mine])
    avg = ensemble_average(curves.astype(np.float64).sum(0), len(mine))
"""
from __future__ import annotations

import heapq

import numpy as np


def partition_members(sizes, world: int) -> list[list[int]]:
    """Splits member indices over ``world`` ranks so that the pair work
    (N(N-1)/2 per member) is balanced: longest-processing-time-first greedy,
    deterministic (ties by rank), so every rank computes the same partition.
    Each rank's list is in ascending member order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = [int(n) for n in sizes]
    order = sorted(range(len(sizes)), key=lambda m: (-sizes[m] * (sizes[m] - 1), m))
    heap = [(0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for m in order:
        load, r = heapq.heappop(heap)
        parts[r].append(m)
        heapq.heappush(heap, (load + sizes[m] * (sizes[m] - 1) // 2, r))
    return [sorted(p) for p in parts]


def partition_loads(sizes, parts) -> list[int]:
    """Pair count of each rank's share."""
    return [sum(int(sizes[m]) * (int(sizes[m]) - 1) // 2 for m in p) for p in parts]


def ensemble_average(local_sum: np.ndarray, local_count: int, group=None) -> np.ndarray:
    """Average curve of the whole ensemble from each rank's FP64 sum of its
    members' curves: one all-reduce of n_q + 1 doubles.  Without an
    initialised process group it is the local average."""
    import torch
    import torch.distributed as dist

    local_sum = np.asarray(local_sum, np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        return local_sum / max(local_count, 1)
    backend = dist.get_backend(group)
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.zeros(len(local_sum) + 1, dtype=torch.float64, device=dev)
    t[:-1] = torch.from_numpy(local_sum).to(dev)
    t[-1] = float(local_count)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t = t.cpu().numpy()
    return t[:-1] / max(t[-1], 1.0)


def combine_shards(local_contrib: np.ndarray, group=None) -> np.ndarray:
    """I(q) of one structure from each rank's ``Debye.calc_shard`` output:
    their sum (one all-reduce of n_q doubles).  Without an initialised
    process group it returns the local contribution."""
    import torch
    import torch.distributed as dist

    local_contrib = np.asarray(local_contrib, np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        return local_contrib
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.from_numpy(local_contrib.copy()).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
