"""Drift windows for the distance cut-off of the time-drift mode
(calc_dc2_drift_, matlab/irc.m:24582-24608), and a plain NumPy FP64
restatement of it used to check the C oracle."""
import math

import numpy as np


def window(n12, n1, nC, n_sites, seed, dup=0):
    rng = np.random.default_rng(seed)
    centres = rng.normal(0, 6, (n_sites, nC))
    s1 = rng.integers(1, n_sites + 1, n12).astype(np.int32)
    s2 = np.where(rng.random(n12) < 0.8, rng.integers(1, n_sites + 1, n12), 0).astype(np.int32)
    F1 = (centres[s1 - 1] + rng.normal(0, 1.5, (n12, nC))).astype(np.float32)
    F2 = (F1 + rng.normal(0, 0.7, (n12, nC))).astype(np.float32)
    if dup:
        F1[1:dup + 1] = F1[0]                    # exact copies: distance 0 (slightly negative in expansion form)
    return F1, F2, s1, s2


def subsample_vr(vi, n_max):
    """subsample_vr_ (matlab/irc.m:11322-11337) on a list of positions."""
    vi = list(vi)
    if len(vi) <= n_max:
        return vi
    n_skip = len(vi) // n_max
    if n_skip > 1:
        vi = vi[::n_skip]
    if len(vi) > n_max:
        n, n_remove = len(vi), len(vi) - n_max
        if n_remove == 1:
            pts = [float(n)]
        else:
            pts = [1.0 + (i * (n - 1.0)) / (n_remove - 1) for i in range(n_remove)]
            pts[0], pts[-1] = 1.0, float(n)
        rm = {min(max(int(math.floor(p + 0.5)), 1), n) for p in pts}
        vi = [v for k, v in enumerate(vi, 1) if k not in rm]
    return vi


def dc2_fp64(n1, s1, s2, F1, F2, n_sites, dc_subsample, dc_percent):
    """The same cut-off with every distance in FP64 (a check of the oracle's
    subsampling, cut index and medians, not of its single-precision bits)."""
    out = []
    for site in range(1, n_sites + 1):
        v11 = subsample_vr(np.flatnonzero(s1[:n1] == site), dc_subsample)
        v21 = subsample_vr(np.flatnonzero(s1 == site), 4 * dc_subsample)
        v22 = subsample_vr(np.flatnonzero(s2 == site), 4 * dc_subsample)
        X = np.concatenate([F1[v21], F2[v22]]).astype(np.float64)
        if not len(v11) or not len(X):
            out.append(np.nan)
            continue
        Y = F1[v11].astype(np.float64)
        D = np.sort(((X[:, None, :] - Y[None, :, :]) ** 2).sum(-1), axis=0)
        cut = int(math.ceil(len(X) * dc_percent / 100.0))
        out.append(np.median(D[cut - 1]))
    out = np.array(out)
    return np.nanmedian(out), out
