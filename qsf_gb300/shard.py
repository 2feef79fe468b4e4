"""Partition independent solves across ranks (one GPU each) with no collective.

A single split-operator solve does not shard without an all-to-all of the FFT
transposes, so multi-GPU runs place whole solves on ranks.  The partition is a
greedy longest-processing-time assignment on the cost m * steps (grid points times
steps): sort by cost, give each solve to the currently least-loaded rank.  It is
deterministic, so every rank computes the same assignment from the same list and
takes its own share -- no data-path communication.  Ranks only meet at the
measurement barrier.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence, Tuple


def cost(points: int, steps: int) -> float:
    return float(points) * float(steps)


def partition(costs: Sequence[float], world_size: int) -> List[List[int]]:
    """Indices of the solves each rank runs (greedy LPT, ties by rank then index)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap: List[Tuple[float, int]] = [(0.0, r) for r in range(world_size)]
    out: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    for lst in out:
        lst.sort()
    return out


def my_share(costs: Sequence[float], world_size: int, rank: int) -> List[int]:
    return partition(costs, world_size)[rank]


def imbalance(costs: Sequence[float], parts: List[List[int]]) -> float:
    """max rank load / mean rank load (1.0 = perfect)."""
    loads = [sum(costs[i] for i in p) for p in parts]
    mean = sum(loads) / len(loads)
    return max(loads) / mean if mean > 0 else 1.0


class StreamAssigner:
    """Online form of the same rule for a request stream: each arriving solve goes to
    the rank with the least cost assigned so far (ties: lowest rank).  Every rank runs
    an assigner over the same ordered stream and keeps the requests assigned to it, so
    the ranks agree without communicating."""

    def __init__(self, world_size: int):
        if world_size < 1:
            raise ValueError("world_size must be >= 1")
        self.loads = [0.0] * world_size

    def assign(self, c: float) -> int:
        r = min(range(len(self.loads)), key=lambda k: (self.loads[k], k))
        self.loads[r] += float(c)
        return r

