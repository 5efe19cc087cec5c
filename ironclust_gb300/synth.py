"""Seeded synthetic spike-feature sites (stand-ins for recorded probes).

The reference measures its clustering stage on SpikeForest hybrid
recordings, which are not available here.  These generators produce sites of
the same shape: Gaussian clusters in D-dimensional feature space plus uniform
noise, cut into equal-count time chunks whose cluster centres drift rigidly
by a random walk, and a drift linkage that joins each chunk to its most
similar chunks within a band (the structure calc_drift_ produces,
matlab/irc2.m:6373-6451).

Named workloads (``WORKLOADS``):

* ``static20k``   20,000 spikes, D=24, 12 clusters, one chunk, knn=30.
* ``drift400k``   400,000 spikes, D=33, 16 clusters, 200 chunks of ~2,000,
                  random-walk drift sd 0.3 per chunk, 15-of-+/-64 linkage, knn=30.
* ``probe10m``    384 sites, 10M spikes (lognormal counts, median 20k, clipped
                  500..200k), D in {18, 24, 33}, 12-40 clusters per site,
                  1,200 chunks, 15-of-+/-64 linkage.
"""
from __future__ import annotations

import numpy as np

from .drift import build_plan, chunk_limits, drift_mask


def make_site(n_spk, n_dim, n_clusters, n_chunks, seed, drift_sd=0.3, drift_slope=0.0,
              noise_frac=0.05, n_link=15, band=64):
    """One site.  Returns dict(F [n_spk, n_dim] float32 (== MATLAB [nC x n]),
    viDrift (0-based chunk id per spike), viLim, mlDrift, centres...)."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 10.0, (n_clusters, n_dim))
    sds = rng.uniform(0.5, 2.0, (n_clusters, n_dim))
    w = rng.dirichlet(np.ones(n_clusters))
    lim = chunk_limits(n_spk, n_chunks)
    chunk = np.repeat(np.arange(n_chunks), np.diff(lim))
    steps = rng.normal(0.0, drift_sd, (n_chunks, n_dim))
    steps[0] = 0.0
    offs = np.cumsum(steps, axis=0) + drift_slope * np.arange(n_chunks)[:, None]
    lab = rng.choice(n_clusters, size=n_spk, p=w)
    F = centres[lab] + offs[chunk] + sds[lab] * rng.standard_normal((n_spk, n_dim))
    n_noise = int(round(noise_frac * n_spk))
    if n_noise:
        lo, hi = F.min(0), F.max(0)
        ii = rng.choice(n_spk, size=n_noise, replace=False)
        F[ii] = rng.uniform(lo, hi, (n_noise, n_dim))
        lab[ii] = -1
    # chunk similarity: -L2 distance between per-chunk centre snapshots (the
    # centres move rigidly, so it is sqrt(K) times the distance of the offsets)
    if n_chunks == 1:
        ml = np.ones((1, 1), bool)
    else:
        mask = (drift_mask(n_chunks, band) if n_chunks > 2 * band + 1 else
                np.abs(np.arange(n_chunks)[None] - np.arange(n_chunks)[:, None]) <= band)
        ml = link_chunks(offs, mask, min(n_link, n_chunks))
    return dict(F=F.astype(np.float32), viDrift=chunk.astype(np.int32), viLim=lim, mlDrift=ml,
                labels=lab.astype(np.int32), n_dim=n_dim)


def link_chunks(offs, mask, n_link):
    """Column j = the n_link chunks nearest chunk j among the masked ones
    (the set dist_mask_ml_ selects; a tie at the n_link-th distance has
    probability zero for a continuous random walk).  Squared distances from
    the Gram matrix, set selection by partition."""
    sq = (offs * offs).sum(1)
    d = sq[:, None] + sq[None, :] - 2.0 * offs @ offs.T
    np.fill_diagonal(d, -1.0)                           # self first, exactly
    d = np.where(mask, d, np.inf)
    mi = np.argpartition(d, n_link - 1, axis=0)[:n_link]
    ml = np.zeros(mask.shape, bool)
    ml[mi, np.arange(mask.shape[1])[None, :]] = True
    return ml


def site_plan(site):
    """Plan over a whole single-page site: every spike is a query."""
    n = site["F"].shape[0]
    return build_plan(site["viDrift"], np.ones(n, bool), site["mlDrift"])


WORKLOADS = {
    "static20k": dict(n_spk=20000, n_dim=24, n_clusters=12, n_chunks=1, seed=1000, knn=30),
    "drift400k": dict(n_spk=400000, n_dim=33, n_clusters=16, n_chunks=200, seed=1001, knn=30),
}


def make_workload(name, scale=1.0, seed_offset=0):
    """A named single-site workload, optionally scaled down in spike count
    (chunk count scaled with it so chunks keep ~2,000 spikes)."""
    cfg = dict(WORKLOADS[name])
    knn = cfg.pop("knn")
    if scale != 1.0:
        cfg["n_spk"] = max(int(cfg["n_spk"] * scale), 200)
        cfg["n_chunks"] = max(1, int(round(cfg["n_chunks"] * scale)))
    cfg["seed"] += seed_offset
    site = make_site(**cfg)
    site["knn"] = knn
    return site


def probe_site_specs(n_sites=384, total=10_000_000, seed=1003, n_chunks=1200):
    """Per-site (n_spk, n_dim, n_clusters) of the probe-scale workload."""
    rng = np.random.default_rng(seed)
    n = np.clip(np.exp(rng.normal(np.log(20000), 1.0, n_sites)), 500, 200000)
    n = np.maximum((n * total / n.sum()).astype(np.int64), 500)
    dims = rng.choice([18, 24, 33], size=n_sites)
    ncl = rng.integers(12, 41, size=n_sites)
    return [dict(n_spk=int(n[i]), n_dim=int(dims[i]), n_clusters=int(ncl[i]),
                 n_chunks=n_chunks, seed=seed * 1000 + i) for i in range(n_sites)]


def make_probe(n_sites=384, total=10_000_000, seed=1003, n_chunks=1200):
    """The probe-scale batch: n_sites sites (lognormal spike counts, D in
    {18, 24, 33}, 12-40 clusters) sharing n_chunks drift chunks."""
    from .batch import SiteBatch
    specs = probe_site_specs(n_sites, total, seed, n_chunks)
    return SiteBatch(make_site(**s) for s in specs), specs
