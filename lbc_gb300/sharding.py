"""Independent cases across ranks: one process per GPU, no data exchange.

The path shards at the level of whole cases (the ducts of a liner sweep, the
requests of a served stream): lbc's solver has no coupling between cases, so
each rank takes a share of the cases, balanced by work (nodes x steps), runs
them on its own GPU as one batch or one server, and only results and timings
travel between ranks, on the host (torch.distributed with the gloo backend).
No collective touches the populations. A single domain larger than one GPU
would need a slab decomposition with a halo exchange per step; one GB300
holds about 3.8 billion nodes in FP32-shifted storage (72 bytes per node for
the two population buffers), so that is not built.
"""
from __future__ import annotations

import heapq
from typing import Callable, List, Sequence


def partition(costs: Sequence[float], world_size: int) -> List[List[int]]:
    """Case indices of every rank: longest-processing-time-first greedy
    (cases by decreasing cost, ties by index, each to the least-loaded rank,
    ties by rank). Deterministic; every index appears exactly once; each
    rank's list is in increasing index order. The largest load exceeds the
    smallest by at most the largest single cost."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world_size)]
    out: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(x) for x in out]


def share(costs: Sequence[float], world_size: int, rank: int) -> List[int]:
    """This rank's case indices (see partition)."""
    if not 0 <= rank < world_size:
        raise ValueError("rank out of range")
    return partition(costs, world_size)[rank]


def loads(costs: Sequence[float], parts: List[List[int]]) -> List[float]:
    return [sum(float(costs[i]) for i in p) for p in parts]


def gather_results(pg, n: int, mine: Sequence[int], results: Sequence) -> list:
    """Every rank's (index, result) pairs gathered on every rank and put back
    in case order: out[i] is the result of case i. pg is torch.distributed (or
    None for one rank)."""
    if len(mine) != len(results):
        raise ValueError("one result per case of this rank")
    pairs = list(zip(mine, results))
    if pg is None:
        allp = [pairs]
    else:
        allp = [None] * pg.get_world_size()
        pg.all_gather_object(allp, pairs)
    out = [None] * n
    seen = 0
    for part in allp:
        for i, r in part:
            if out[i] is not None:
                raise RuntimeError(f"case {i} returned by two ranks")
            out[i] = r
            seen += 1
    if seen != n:
        raise RuntimeError(f"{n - seen} cases were not run by any rank")
    return out


def run_sharded(items: Sequence, costs: Sequence[float], fn: Callable[[list], list], pg=None) -> list:
    """Run fn on this rank's share of items (fn takes a list, returns one
    result per item in order) and return all results in item order on every
    rank."""
    ws = pg.get_world_size() if pg is not None else 1
    rank = pg.get_rank() if pg is not None else 0
    mine = share(costs, ws, rank)
    res = fn([items[i] for i in mine]) if mine else []
    return gather_results(pg, len(items), mine, list(res))


def all_max(pg, x: float) -> float:
    """Largest x over ranks (x itself for one rank)."""
    if pg is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def all_sum(pg, x: float) -> float:
    """Sum of x over ranks (x itself for one rank)."""
    if pg is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())
