"""Drift-linkage encoding, paging and per-chunk launch plans (host side,
numpy).  The linkage itself (calc_drift_) runs on the device: irc.calc_drift.

Mirrors the irc2 host logic that sits around the hot-path kernels:

* ``mi2ml_drift``       mi2ml_drift_       matlab/irc2.m:6509-6516
* ``drift_mask``        the chunk band calc_drift_ searches above
                        nTime_max_drift chunks, matlab/irc2.m:6425-6431
* ``plan_sort_page``    plan_sort_page_    matlab/irc2.m:3914-3946
* ``build_plan``        the per-chunk run selection inside search_knn_drift_ /
                        search_delta_drift_, matlab/irc2.m:3752-3760,
                        :3764-3773 and :3808-3812, :3829-3837

Indices are 0-based here; chunk ids are 0-based (MATLAB's discretize gives
1-based ids, the shift is applied at the MEX/MATLAB boundary only).

A *plan* is the compact description of every kernel launch the MATLAB loop
would make for one site: for query chunk i, queries ``[q0[i], q0[i]+nq[i])``
(positions in the site feature matrix) and candidate runs
``rs[roff[i]:roff[i+1]]`` / ``rn[...]`` (0-based run start and length; the
IBB/NBB arguments of search_min_drift).  Outputs are indexed by
``q - q_base`` with ``n_out`` rows.
"""
from __future__ import annotations

import math

import numpy as np


def matlab_round(x):
    """MATLAB round: halves away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def mi2ml_drift(mi_member):
    """mi2ml_drift_: column j of the result marks the chunks listed in column j."""
    mi_member = np.asarray(mi_member)
    n_members, n_drift = mi_member.shape
    ml = np.zeros((n_drift, n_drift), bool)
    ml[mi_member.ravel(order="F"), np.repeat(np.arange(n_drift), n_members)] = True
    return ml


def drift_mask(n_drift, quarter):
    """The |i-j| <= quarter band with the edge blocks calc_drift_ adds
    (matlab/irc2.m:6425-6431)."""
    i = np.arange(n_drift)
    m = np.abs(i[None, :] - i[:, None]) <= quarter
    m[: quarter * 2 + 1, :quarter] = True
    m[-(quarter * 2 + 1):, -quarter:] = True
    return m


def plan_sort_page(nTime_drift, viLim_drift, nTime_max_drift=256):
    """plan_sort_page_ (matlab/irc2.m:3914-3946), 0-based.

    Returns a list of pages: dict(drift_out=(a, b), drift_in=(a, b),
    spk_out=(s0, s1), spk_in=(s0, s1)) with inclusive chunk ranges and
    half-open spike ranges."""
    n = nTime_drift
    width = nTime_max_drift
    quarter, half = width // 4, width // 2
    n_pages = n // half
    lim = np.asarray(viLim_drift)
    if n_pages == 0:
        return [dict(drift_out=(0, n - 1), drift_in=(0, n - 1),
                     spk_out=(int(lim[0]), int(lim[-1])), spk_in=(int(lim[0]), int(lim[-1])))]
    pages, ib_prev = [], 0
    for p in range(1, n_pages + 1):
        iB = min((p - 1) * half + width, n)
        iA = max(1, iB - width + 1)
        ia = 1 if p == 1 else min(iA + quarter, n)
        ia = max(ib_prev + 1, ia)
        ib = n if p == n_pages else max(iB - quarter, 1)
        ib_prev = ib
        pages.append(dict(drift_out=(iA - 1, iB - 1), drift_in=(ia - 1, ib - 1),
                          spk_out=(int(lim[iA - 1]), int(lim[iB])),
                          spk_in=(int(lim[ia - 1]), int(lim[ib]))))
    return pages


def build_plan(viDrift_out, vl_in, mlDrift):
    """Per-chunk launch plan of search_knn_drift_ (matlab/irc2.m:3752-3787).

    viDrift_out: chunk id of every column of the site feature matrix (primary
    spikes sorted by time, then optional secondary-site copies).  vl_in:
    boolean mask of the query columns (a contiguous range).  mlDrift: [nDrift
    x nDrift] boolean; column a lists the chunks linked to chunk a."""
    vd = np.asarray(viDrift_out).astype(np.int64).ravel()
    vl = np.asarray(vl_in).astype(bool).ravel()
    ml = np.asarray(mlDrift).astype(bool)
    if not vl.any():
        raise ValueError("build_plan: no query spikes")
    in_idx = np.flatnonzero(vl)
    in_offset = int(in_idx[0])
    if in_idx[-1] - in_offset + 1 != in_idx.size:
        raise ValueError("build_plan: query columns must be contiguous")
    vd_in = vd[vl]
    change = np.flatnonzero(np.diff(vd)) + 1
    viiBB = np.concatenate([[0], change, [vd.size]]).astype(np.int64)
    viBB = vd[viiBB[:-1]]
    vnBB = np.diff(viiBB)
    # query chunks present in the in-set, in increasing chunk id
    chunks, first, count = np.unique(vd_in, return_index=True, return_counts=True)
    last = np.unique(vd_in[::-1], return_index=True)[1]
    last = vd_in.size - 1 - last
    if np.any(last - first + 1 != count):
        bad = int(chunks[np.flatnonzero(last - first + 1 != count)[0]])
        raise ValueError("build_plan: chunk %d queries are not contiguous" % bad)
    # runs linked to every query chunk, in run order (ml[:, a] of each run's chunk)
    link = ml[np.ix_(viBB, chunks)].T                      # [n query chunks x n runs]
    a_idx, r_idx = np.nonzero(link)
    roff = np.concatenate([[0], np.cumsum(np.bincount(a_idx, minlength=chunks.size))])
    i32 = lambda v: np.asarray(v, np.int32)
    return dict(q0=i32(first + in_offset), nq=i32(count), roff=i32(roff), rs=i32(viiBB[r_idx]),
                rn=i32(vnBB[r_idx]), q_base=in_offset, n_out=int(vl.sum()), n_f=int(vd.size))


def plan_pairs(plan):
    """Number of (query, candidate) pairs the plan evaluates."""
    roff, rn, nq = plan["roff"], plan["rn"].astype(np.int64), plan["nq"].astype(np.int64)
    per_chunk = np.array([rn[roff[i]:roff[i + 1]].sum() for i in range(len(nq))], np.int64)
    return int((per_chunk * nq).sum())


def plan_chunk(plan, i):
    """(IBB, NBB, vnConst-without-nC/nF) of query chunk i."""
    r0, r1 = int(plan["roff"][i]), int(plan["roff"][i + 1])
    return plan["rs"][r0:r1], plan["rn"][r0:r1], int(plan["q0"][i]), int(plan["nq"][i])


def chunk_limits(n_spk, n_chunks):
    """Equal-count chunk limits, 0-based: ceil((1:n)/n * N) (matlab/irc2.m:6395)."""
    return np.concatenate([[0], [math.ceil(i / n_chunks * n_spk) for i in range(1, n_chunks + 1)]]).astype(np.int64)
