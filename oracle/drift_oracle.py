"""numpy restatement of calc_drift_ (matlab/irc2.m:6373-6465): TEST
INFRASTRUCTURE ONLY, the checker of the device linkage irc_calc_drift.
Only tests/ import it.

* ``subsample_vr``  subsample_vr_   matlab/irc2.m:1557-1573
* ``quantile_vr``   quantile_vr_    matlab/irc2.m:6481-6490
* ``histcounts2``   MATLAB histcounts2 (bins [e_i, e_i+1), the last closed)
* ``dist_mask_ml``  dist_mask_ml_   matlab/irc2.m:6455-6465
* ``calc_drift``    calc_drift_     matlab/irc2.m:6373-6451 (without its parfor
                                    and plot branches)

Distances are computed in float64 from integer counts, which is exact, so
the chunk order equals the order of the true distances.  MATLAB's pdist and
sort on single data are closed code: their rounding is restated, not pinned.
"""
from __future__ import annotations

import numpy as np


def matlab_round(x):
    """MATLAB round: halves away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def mi2ml_drift(mi_member):
    mi_member = np.asarray(mi_member)
    n_members, n_drift = mi_member.shape
    ml = np.zeros((n_drift, n_drift), bool)
    ml[mi_member.ravel(order="F"), np.repeat(np.arange(n_drift), n_members)] = True
    return ml


def drift_mask(n_drift, quarter):
    i = np.arange(n_drift)
    m = np.abs(i[None, :] - i[:, None]) <= quarter
    m[: quarter * 2 + 1, :quarter] = True
    m[-(quarter * 2 + 1):, -quarter:] = True
    return m


def subsample_vr(vi, n_max):
    """subsample_vr_ (matlab/irc2.m:1557-1573)."""
    vi = np.asarray(vi)
    if vi.size > n_max:
        n_skip = vi.size // n_max
        if n_skip > 1:
            vi = vi[::n_skip]
        if vi.size > n_max:
            n_remove = vi.size - n_max
            rm = matlab_round(np.linspace(1, vi.size, n_remove)).astype(np.int64)
            rm = np.clip(rm, 1, vi.size) - 1
            keep = np.ones(vi.size, bool)
            keep[rm] = False
            vi = vi[keep]
    return vi




def quantile_vr(vr, vr_q, max_sample=100000):
    """quantile_vr_ (matlab/irc2.m:6481-6490)."""
    vr = subsample_vr(np.asarray(vr), max_sample)
    n = vr.size
    idx = np.maximum(np.minimum(matlab_round(n * np.asarray(vr_q, np.float64)), n), 1).astype(np.int64)
    return np.sort(vr, kind="stable")[idx - 1]




def histcounts2(x, y, xedges, yedges):
    """MATLAB histcounts2: bins [e_i, e_{i+1}), the last bin closed."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    xe = np.asarray(xedges, np.float64)
    ye = np.asarray(yedges, np.float64)
    nx, ny = xe.size - 1, ye.size - 1
    ix = np.searchsorted(xe, x, side="right") - 1
    iy = np.searchsorted(ye, y, side="right") - 1
    ix[x == xe[-1]] = nx - 1
    iy[y == ye[-1]] = ny - 1
    ok = (ix >= 0) & (ix < nx) & (iy >= 0) & (iy < ny) & (x >= xe[0]) & (y >= ye[0])
    out = np.zeros((nx, ny), np.float64)
    np.add.at(out, (ix[ok], iy[ok]), 1)
    return out




def dist_mask_ml(mrF, ml_mask, nneigh):
    """dist_mask_ml_: per column, the nneigh nearest masked columns of mrF
    (Euclidean, stable ascending sort).  mrF: [nFeat, nDrift]."""
    mrF = np.asarray(mrF, np.float64)
    n = mrF.shape[1]
    ml = np.zeros((n, n), bool)
    for j in range(n):
        rows = np.flatnonzero(ml_mask[:, j])
        d = np.sqrt(((mrF[:, [j]] - mrF[:, rows]) ** 2).sum(0))
        srt = np.argsort(d, kind="stable")
        ml[rows[srt[:nneigh]], j] = True
    return ml




def calc_drift(vrAmp_spk, vrPos_spk, n_sites, nTime_drift, nTime_batch, nTime_max_drift=256,
               nQuantile_drift=10):
    """calc_drift_ (matlab/irc2.m:6373-6451) without its parfor/plot branches.

    Returns (viLim_drift, mlDrift): 0-based chunk limits [nTime_drift+1]
    (chunk i = spikes viLim[i]..viLim[i+1]-1) and the linkage matrix.
    """
    n_spk = len(vrAmp_spk)
    if not nTime_batch or not nTime_drift or nTime_batch >= nTime_drift:
        return np.array([0, n_spk], np.int64), np.ones((1, 1), bool)
    lim = np.concatenate([[0], np.ceil(np.arange(1, nTime_drift + 1) / nTime_drift * n_spk)]).astype(np.int64)
    amp = np.asarray(vrAmp_spk, np.float32)
    pos = np.asarray(vrPos_spk, np.float32)
    amp_q = quantile_vr(amp, np.arange(nQuantile_drift + 1) / nQuantile_drift)
    pos_q = quantile_vr(pos, np.arange(n_sites + 1) / n_sites)
    counts = np.zeros((nQuantile_drift * n_sites, nTime_drift), np.float32)
    for i in range(nTime_drift):
        h = histcounts2(amp[lim[i]:lim[i + 1]], pos[lim[i]:lim[i + 1]], amp_q, pos_q)
        counts[:, i] = h.ravel(order="F")
    if nTime_drift > nTime_max_drift:
        quarter = nTime_max_drift // 4
        ml = dist_mask_ml(counts, drift_mask(nTime_drift, quarter), nTime_batch)
    else:
        d = np.sqrt(((counts[:, :, None] - counts[:, None, :]).astype(np.float64) ** 2).sum(0))
        mi = np.argsort(d, axis=0, kind="stable")[:nTime_batch, :]
        ml = mi2ml_drift(mi)
    return lim, ml
