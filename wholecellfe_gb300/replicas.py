"""Multi-GPU host logic: a population of independent cells sharded over ranks.

Cells never exchange data during a step (each cell's step reads only its own
mesh, state and substrate, cellBP/UL_growth_explicit.cpp:2016-2121), so the
multi-GPU form is one engine per rank over a disjoint shard of the cells, with
no collective on the data path.  The only collectives are host-side: a barrier
around the timed region and a max over ranks of the elapsed time.

Sharding balances the per-rank work, which is proportional to the vertex (and
triangle) count: longest-processing-time first, ties broken by cell index, so
that every rank computes the same assignment without communicating.
"""
from __future__ import annotations

import heapq
import os
from dataclasses import dataclass


@dataclass(frozen=True)
class RankEnv:
    rank: int
    world: int
    local: int


def rank_env(env=None) -> RankEnv:
    """RANK / WORLD_SIZE / LOCAL_RANK as set by torch.distributed.run (1 rank when unset)."""
    env = os.environ if env is None else env
    world = int(env.get("WORLD_SIZE", "1"))
    rank = int(env.get("RANK", "0"))
    local = int(env.get("LOCAL_RANK", str(rank)))
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of world {world}")
    return RankEnv(rank, world, local)


def partition_cells(costs, world: int) -> list[list[int]]:
    """Assign cell indices to `world` ranks, balancing the summed cost.

    Greedy LPT: cells in decreasing cost (equal costs by increasing index) go to
    the rank with the smallest load so far (equal loads by increasing rank).
    Deterministic; every index appears exactly once; each rank's list is sorted.
    The largest load is at most 4/3 of the optimum plus one cell."""
    if world < 1:
        raise ValueError("world must be >= 1")
    costs = [float(c) for c in costs]
    if any(c < 0 for c in costs):
        raise ValueError("costs must be non-negative")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in shards]


def shard_loads(costs, shards) -> list[float]:
    return [float(sum(costs[i] for i in s)) for s in shards]


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest `value` over all ranks (the job time of a timed region)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device=None) -> float:
    """The sum of `value` over all ranks (units processed by the whole job)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
