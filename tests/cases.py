"""Seeded test sites with the edge cases the reference kernels meet.

* exact duplicate spikes (squared distance 0: dropped by the irc2 kernels,
  kept by cuda_knn_index / cuda_delta_knn);
* ragged chunks (query counts not a multiple of any tile size, a chunk of a
  single spike, chunks with fewer candidates than knn);
* run counts that do not divide the bin count (the reference's duplicated
  "extra" bins);
* secondary-site feature copies appended after the primary spikes
  (two runs per linked chunk, matlab/irc2.m:3892-3897);
* rho ties (the strict rho mask of the delta kernels).
"""
from __future__ import annotations

import numpy as np

from ironclust_gb300 import synth
from ironclust_gb300.drift import build_plan


def small_site(n=3000, d=24, n_chunks=5, seed=7, n_dup=40, secondary=False, sizes=None):
    """A site with duplicates; returns (F [nF, d] float32, plan dict, viDrift)."""
    rng = np.random.default_rng(seed)
    s = synth.make_site(n, d, 6, n_chunks, seed)
    F = s["F"].copy()
    vd = s["viDrift"].copy()
    if sizes is not None:                           # ragged chunk sizes
        lim = np.concatenate([[0], np.cumsum(sizes)])
        assert lim[-1] == n
        vd = np.repeat(np.arange(len(sizes)), sizes).astype(np.int32)
    # exact duplicates inside chunks
    for _ in range(n_dup):
        i = int(rng.integers(0, n - 1))
        j = i + 1
        if vd[i] == vd[j]:
            F[j] = F[i]
    ml = s["mlDrift"] if sizes is None else _band_links(len(sizes))
    vl = np.ones(n, bool)
    if secondary:
        # append secondary-site copies of 1/3 of the spikes (time order kept)
        pick = np.sort(rng.choice(n, size=n // 3, replace=False))
        F2 = F[pick] + rng.normal(0, 0.5, (pick.size, d)).astype(np.float32)
        F = np.concatenate([F, F2]).astype(np.float32)
        vd = np.concatenate([vd, vd[pick]]).astype(np.int32)
        vl = np.concatenate([vl, np.zeros(pick.size, bool)])
    plan = build_plan(vd, vl, ml)
    return F, plan, vd


def _band_links(n_chunks, k=3):
    ml = np.zeros((n_chunks, n_chunks), bool)
    for j in range(n_chunks):
        for i in range(max(0, j - k // 2), min(n_chunks, j + k // 2 + 1)):
            ml[i, j] = True
    return ml


def rho_with_ties(n, seed=3):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.1, 1.0, n).astype(np.float32)
    r[rng.choice(n, n // 10, replace=False)] = np.float32(0.5)     # a tie group
    return r
