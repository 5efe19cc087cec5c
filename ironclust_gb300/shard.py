"""Site sharding across ranks (one process per GPU).

Every probe site's kNN, rho and delta read only that site's features and rho
(matlab/irc2.m:3535-3561, the parfor over sites), so sites are independent
units: they are split over ranks with no exchange of data.  Sites go to the
least-loaded rank in decreasing order of cost (longest-processing-time
first), the cost of a site being its (query, candidate) pair count times its
feature dimension.
"""
from __future__ import annotations

import heapq


def site_cost(pairs, n_dim):
    return int(pairs) * int(n_dim)


def assign_sites(costs, world_size):
    """LPT assignment: returns a list of site-index lists, one per rank.
    Deterministic (ties by site index, then rank)."""
    if world_size <= 0:
        raise ValueError("world_size must be positive")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0, r) for r in range(world_size)]
    out = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    for lst in out:
        lst.sort()
    return out


def rank_sites(costs, rank, world_size):
    return assign_sites(costs, world_size)[rank]


def imbalance(costs, assignment):
    loads = [sum(costs[i] for i in s) for s in assignment]
    mean = sum(loads) / len(loads)
    return max(loads) / mean if mean else 1.0
