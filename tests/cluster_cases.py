"""Inputs for the clustering step after the path, and a literal pure-Python
restatement of it used to cross-check the C oracle on small cases.

The restatement follows the MATLAB text line by line with Python lists:
postCluster_ / assignCluster_knn_ (matlab/irc2.m:6520-6535, :6640-6694),
cell2map_ (:6754-6805), dpclus_remove_count_ (:6735-6750) and the output
normalisation of sort_ (:3263-3264).
"""
from __future__ import annotations

import math

import numpy as np


def _desc_order(x):
    """sort(x, 'descend') order, 0-based: NaN first, stable."""
    return sorted(range(len(x)), key=lambda i: (0, 0.0) if math.isnan(x[i]) else (1, -float(x[i])))


def sort_rho_literal(rho):
    r = np.asarray(rho, np.float32)
    ok = r[~np.isnan(r)]
    m = np.float32(ok.max()) if ok.size else np.float32(np.nan)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = (r / m).astype(np.float32)
    return r, np.array(_desc_order(list(r)), np.int64) + 1


def assign_cluster_knn_literal(rho, delta, ordrho, nneigh, miKnn, delta_cut=1.0, min_count=0):
    rho = [np.float32(x) for x in rho]
    delta = [np.float32(x) for x in delta]
    ordrho = [int(x) for x in ordrho]
    nneigh = [int(x) for x in nneigh]
    mk = [[int(v) for v in row] for row in np.asarray(miKnn)]
    nSpk = len(rho)
    cut = np.float32(delta_cut)
    # viSpk_peak = find(vrDelta_spk(:) >= delta_cut)
    peaks = [s + 1 for s in range(nSpk) if delta[s] >= cut]
    nClu_pre = len(peaks)
    viClu = [0] * nSpk
    # [vrRho_peak, ix_] = sort(vrRho_spk(viSpk_peak), 'descend')
    order = _desc_order([rho[p - 1] for p in peaks])
    peaks = [peaks[i] for i in order]
    # cvi_peak{i} = find(any(ismember(miKnn_peak, miKnn_peak(:,i))))'
    cols = [mk[p - 1] for p in peaks]
    cvi = []
    for i in range(len(peaks)):
        ci = set(cols[i])
        cvi.append([j + 1 for j in range(len(peaks)) if any(v in ci for v in cols[j])])
    # cell2map_
    nClu = len(cvi)
    for _ in range(10):
        cvi1 = [[] for _ in range(nClu)]
        for iClu in [i for i in range(nClu) if len(cvi[i]) > 1]:
            v = list(cvi[iClu])
            for m in cvi[iClu]:
                v += cvi[m - 1]
            v = sorted(set(v))
            for m in v:
                cvi1[m - 1] = v
        if all(len(a) == len(b) for a, b in zip(cvi1, cvi)):
            break
        cvi = cvi1
    viMapClu = [min(c) if c else i + 1 for i, c in enumerate(cvi)]
    uniq = sorted(set(viMapClu) - {0})
    rank = {r: k + 1 for k, r in enumerate(uniq)}
    for i, p in enumerate(peaks):
        viClu[p - 1] = rank[viMapClu[i]]
    icl = [peaks[u - 1] for u in uniq]
    if len(icl) <= 1:
        viClu = [1] * nSpk
        icl = [ordrho[0]]
    else:
        nneigh1 = [nneigh[o - 1] for o in ordrho]
        for _ in range(10):
            vi = [ii for ii in range(nSpk) if viClu[ordrho[ii] - 1] <= 0]
            if not vi:
                break
            for ii in vi:
                viClu[ordrho[ii] - 1] = viClu[nneigh1[ii] - 1]
            if sum(1 for x in viClu if x <= 0) == 0:
                break
    nClu_post = len(icl)
    # dpclus_remove_count_
    cnt = [0] * (nClu_post + 1)
    for x in viClu:
        if 1 <= x <= nClu_post:
            cnt[x] += 1
    keep = [cnt[c] >= min_count for c in range(1, nClu_post + 1)]
    vn = cnt[1:]
    if not all(keep):
        viMap = [0] * (nClu_post + 1)
        k = 0
        for c in range(1, nClu_post + 1):
            if keep[c - 1]:
                k += 1
                viMap[c] = k
        viClu = [viMap[x] if 1 <= x <= nClu_post else 0 for x in viClu]
        icl = [icl[c] for c in range(nClu_post) if keep[c]]
        vn = [vn[c] for c in range(nClu_post) if keep[c]]
    return dict(viClu=np.array(viClu, np.int32), icl=np.array(icl, np.int64),
                vnSpk_clu=np.array(vn, np.int32), nClu=len(icl), nClu_pre=nClu_pre, nClu_post=nClu_post)


def random_case(seed, n=400, knn=6, vocab=None, levels=None, p_quirk=0.05, p_nan=0.0,
                delta_scale=1.5):
    """A synthetic clustering input with the shapes of the real one.

    rho (optionally quantised to ``levels`` values, so ties occur), delta
    (optionally with NaN), ordrho from the MATLAB order, nneigh pointing to a
    spike earlier in ordrho, except a ``p_quirk`` share that points anywhere
    (later spikes, itself), and kNN lists drawn from ``vocab`` ids so that
    peak lists overlap.  Returns raw (unnormalised) rho; callers normalise."""
    rng = np.random.default_rng(seed)
    rho = rng.gamma(2.0, 1.0, n).astype(np.float32)
    if levels:
        rho = (np.round(rho * levels) / levels + 0.01).astype(np.float32)
    if p_nan:
        rho[rng.random(n) < p_nan] = np.nan
    delta = (rng.exponential(delta_scale, n) * rng.random(n) * 1.2).astype(np.float32)
    if p_nan:
        delta[rng.random(n) < p_nan] = np.nan
    rn, ordrho = sort_rho_literal(rho)
    pos = np.empty(n, np.int64)
    pos[ordrho - 1] = np.arange(n)
    nneigh = np.empty(n, np.int64)
    for s in range(n):
        r = pos[s]
        if r == 0 or rng.random() < p_quirk:
            nneigh[s] = rng.integers(1, n + 1)
        else:
            nneigh[s] = ordrho[rng.integers(0, r)]
    V = vocab or n
    miKnn = rng.integers(1, V + 1, size=(n, knn)).astype(np.int64)
    miKnn[:, 0] = np.arange(1, n + 1)           # self first, as the kNN lists hold
    return rn, delta, ordrho, nneigh, miKnn


def geometric_case(seed, n=3000, dim=4, n_clusters=6, knn=12):
    """kNN, rho, delta and nneigh computed from Gaussian blobs in float64, as
    the path would produce them (delta = distance to the nearest higher-rho
    spike over the kNN distance, top spike -> sqrt(SINGLE_INF) * rho)."""
    rng = np.random.default_rng(seed)
    cen = rng.normal(0, 6, (n_clusters, dim))
    lab = rng.integers(0, n_clusters, n)
    X = cen[lab] + rng.normal(0, 1, (n, dim))
    d2 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    nb = np.argsort(d2, axis=1, kind="stable")[:, :knn]
    dk = np.sqrt(d2[np.arange(n), nb[:, -1]])
    rho = (1.0 / dk).astype(np.float32)
    delta = np.empty(n, np.float32)
    nneigh = np.empty(n, np.int64)
    for i in range(n):
        hi = np.nonzero(rho > rho[i])[0]
        if hi.size == 0:
            delta[i] = np.float32(math.sqrt(3.402e38)) * rho[i]
            nneigh[i] = i + 1
        else:
            j = hi[np.argmin(d2[i, hi])]
            delta[i] = np.float32(math.sqrt(d2[i, j])) * rho[i]
            nneigh[i] = j + 1
    rn, ordrho = sort_rho_literal(rho)
    return rn, delta, ordrho, nneigh, (nb + 1).astype(np.int64)
