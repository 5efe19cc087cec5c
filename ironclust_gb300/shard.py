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


# ---------------------------------------------------------------------------
# A probe's sites over ranks: each rank runs the library on the sub-batch of
# its share; rank 0 puts the shares' outputs back in the batch's spike order.
# ---------------------------------------------------------------------------

ID_KEYS = ("miKnn", "nneigh")      # outputs holding 1-based spike ids of the batch


def batch_costs(batch):
    """site_cost of every site of a SiteBatch."""
    from .drift import plan_pairs
    return [site_cost(plan_pairs(p), d) for p, d in zip(batch.site_plans, batch.dims)]


def batch_share(batch, rank, world_size):
    """(site indices, SiteBatch) of rank's LPT share of the batch's sites."""
    idx = rank_sites(batch_costs(batch), rank, world_size)
    return idx, batch.subset(idx)


def merge_shares(batch, shares):
    """Outputs of the whole batch from its shares.

    shares: [(site indices, outputs)], outputs a dict of arrays whose rows are
    the spikes of that share's sub-batch (its sites stacked in the order of
    the indices).  Rows go to the sites' rows of the batch; the spike ids in
    ID_KEYS (1-based, always ids of the same site) are moved by the site's
    offset.  Every site must be in exactly one share."""
    import numpy as np
    seen = np.zeros(batch.n_sites, np.int32)
    merged = {}
    for idx, out in shares:
        idx = [int(i) for i in idx]
        seen[idx] += 1
        sub_bases = np.concatenate([[0], np.cumsum(batch.sizes[idx])]).astype(np.int64)
        for key, a in out.items():
            if a is None:
                continue
            a = np.asarray(a)
            if a.shape[0] != sub_bases[-1]:
                raise ValueError("merge_shares: %s has %d rows, the share %d spikes" % (key, a.shape[0],
                                                                                      sub_bases[-1]))
            dst = merged.get(key)
            if dst is None:
                dst = merged[key] = np.zeros((int(batch.bases[-1]),) + a.shape[1:], a.dtype)
            for j, s in enumerate(idx):
                rows = a[sub_bases[j]:sub_bases[j + 1]]
                if key in ID_KEYS:
                    shift = int(batch.bases[s] - sub_bases[j])
                    rows = np.where(rows > 0, rows + shift, rows).astype(a.dtype)
                dst[batch.site_slice(s)] = rows
    if not np.all(seen == 1):
        raise ValueError("merge_shares: sites %s are not in exactly one share" % np.flatnonzero(seen != 1)[:8])
    return merged


def gather_merge(batch, idx, out, rank, world_size, group=None):
    """Send this rank's (site indices, host outputs) to rank 0 over a CPU
    (gloo) process group; rank 0 returns the merged outputs of the whole
    batch, the other ranks None.  This collects results after the work; no
    rank waits on another's data while it computes."""
    import torch.distributed as dist
    parts = [None] * world_size if rank == 0 else None
    dist.gather_object((list(idx), out), parts, dst=0, group=group)
    return merge_shares(batch, parts) if rank == 0 else None
