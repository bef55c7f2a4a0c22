"""Sharding the batching form over GPUs (one rank per GPU).

Independent systems need no exchange: each rank steps a contiguous range of
the systems in its own context, and only the timing is reduced (max over
ranks). The reference steps one scene on one device and queue
(Astro/Renderer.swift:115-117); this has no counterpart there.

The ranges balance the step's cost, which grows like N log N per system
(the sort and the tree depth go as log N, the walk per particle as log N):
the contiguous partition minimising the largest rank's sum of
N_s log2(max(N_s, 2)), found exactly by a binary search on that largest sum
with a greedy fill. Its largest sum is at most total / world + the largest
single system's cost (a greedy fill at that bound always fits).
"""
from __future__ import annotations

import math


def system_cost(n: int) -> float:
    """Relative cost of stepping a system of n particles: n log2 n."""
    return float(n) * math.log2(max(int(n), 2))


def _fits(costs, world: int, cap: float) -> bool:
    parts, acc = 1, 0.0
    for c in costs:
        if c > cap:
            return False
        if acc + c > cap:
            parts += 1
            acc = c
            if parts > world:
                return False
        else:
            acc += c
    return True


def partition_systems(sizes, world: int) -> list[tuple[int, int]]:
    """Contiguous system ranges [begin, end) for ranks 0..world-1 (a rank may
    get an empty range when there are fewer systems than ranks), minimising
    the largest rank cost."""
    if world < 1:
        raise ValueError("world must be >= 1")
    costs = [system_cost(int(s)) for s in sizes]
    if not costs:
        return [(0, 0)] * world
    lo, hi = max(costs), sum(costs)
    for _ in range(100):  # binary search on the largest rank cost
        mid = 0.5 * (lo + hi)
        if _fits(costs, world, mid):
            hi = mid
        else:
            lo = mid
        if hi - lo <= 1e-9 * hi:
            break
    ranges, begin, acc = [], 0, 0.0
    for i, c in enumerate(costs):
        if acc + c > hi and i > begin:
            ranges.append((begin, i))
            begin, acc = i, 0.0
        acc += c
    ranges.append((begin, len(costs)))
    while len(ranges) < world:
        ranges.append((len(costs), len(costs)))
    return ranges


def rank_cost(sizes, rng) -> float:
    return sum(system_cost(int(s)) for s in sizes[rng[0]:rng[1]])


def particle_range(sizes, rng) -> tuple[int, int]:
    """First and end particle of a system range (systems back to back)."""
    first = sum(int(s) for s in sizes[:rng[0]])
    return first, first + sum(int(s) for s in sizes[rng[0]:rng[1]])
