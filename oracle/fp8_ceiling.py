"""Recall ceiling of an FP8-e4m3 distance filter (ANALYSIS / TEST
INFRASTRUCTURE: not part of the library; run by hand or by the tests).

The FP8 form's tensor-core filter ranks candidates by the squared distance
between e4m3-quantised feature vectors, |Q(s(a - ref)) - Q(s(b - ref))|^2,
and hands the best candidates to the exact FP32 re-rank.  A true neighbour
ranked outside the handed-over list is lost whatever the re-rank does, so
the recall of the form is bounded by

    ceiling(M) = fraction of the FP64 k nearest that lie among the M nearest
                 by the quantised distance,

M being the list length (the filter hands over ~70-90 candidates per query;
BASELINE's precision form names a 60-candidate over-fetch).  This module
measures that ceiling on a sample of queries of a workload for three
quantisations:

  global    one scale s = 32 / max|F - ref| for the whole site (the form's
            scaling: ref = the mean of the site's queries);
  per_pair  per-(query chunk, candidate chunk) absmax scaling: both chunks'
            rows scaled by 32 / max(max|F_q - ref|, max|F_c - ref|), so
            the MMA result stays a known multiple of the distance;
  centred   per query chunk centring: ref = the query chunk's mean for that
            chunk's candidates as well (distances unchanged, operand
            magnitudes smaller).

e4m3 is emulated exactly in numpy: round-to-nearest-even to 3 mantissa bits,
normal exponents -6..8, subnormal step 2^-9, saturation at 448.  A power-of-
two or any other scale changes the relative precision of normal e4m3 values
not at all, so absmax scaling alone cannot raise the ceiling; only smaller
operand magnitudes relative to the neighbour distances (centring) can.
"""
from __future__ import annotations

import numpy as np


def e4m3(x):
    """Round to the nearest e4m3 value (ties to even), saturating at +-448."""
    x = np.asarray(x, np.float64)
    a = np.abs(x)
    e = np.floor(np.log2(np.maximum(a, 2.0 ** -9)))
    e = np.clip(e, -6, 8)
    step = 2.0 ** (e - 3)
    q = np.minimum(np.round(a / step) * step, 448.0)
    return np.sign(x) * q


def _chunk_rows(plan, i):
    q0, nq = int(plan["q0"][i]), int(plan["nq"][i])
    a, b = int(plan["roff"][i]), int(plan["roff"][i + 1])
    runs = [(int(plan["rs"][r]), int(plan["rn"][r])) for r in range(a, b)]
    return np.arange(q0, q0 + nq), runs


def ceiling(F, plan, knn=30, Ms=(60, 90, 128, 192), chunks=None, queries_per_chunk=64, seed=7):
    """dict(mode -> {M: ceiling}) over a sample of queries (queries_per_chunk
    from each of `chunks`, default 8 evenly spaced query chunks)."""
    F = np.asarray(F, np.float64)
    n_ch = len(plan["q0"])
    if chunks is None:
        chunks = np.unique(np.linspace(0, n_ch - 1, min(8, n_ch)).astype(int))
    rng = np.random.default_rng(seed)
    ref = F.mean(0)
    s_glob = 32.0 / np.abs(F - ref).max()
    hits = {m: {M: 0 for M in Ms} for m in ("global", "per_pair", "centred")}
    total = 0
    for i in chunks:
        qrows, runs = _chunk_rows(plan, int(i))
        if len(qrows) == 0:
            continue
        qs = np.sort(rng.choice(qrows, size=min(queries_per_chunk, len(qrows)), replace=False))
        cand = np.concatenate([np.arange(s, s + n) for s, n in runs])
        A, B = F[qs], F[cand]
        d64 = ((A[:, None, :] - B[None, :, :]) ** 2).sum(-1)
        d64[d64 <= 0] = np.inf                        # the reference excludes distance 0
        true = np.argsort(d64, axis=1, kind="stable")[:, :knn]
        # quantised distances per mode
        qa = e4m3(s_glob * (A - ref))
        qb = e4m3(s_glob * (B - ref))
        dq = {"global": ((qa[:, None, :] - qb[None, :, :]) ** 2).sum(-1)}
        mq = np.abs(F[qrows] - ref).max()
        parts = []
        for s0, n in runs:
            Bc = F[s0:s0 + n]
            sp = 32.0 / max(mq, np.abs(Bc - ref).max())
            qa_p, qb_p = e4m3(sp * (A - ref)), e4m3(sp * (Bc - ref))
            parts.append(((qa_p[:, None, :] - qb_p[None, :, :]) ** 2).sum(-1) / sp ** 2)
        dq["per_pair"] = np.concatenate(parts, axis=1)
        cref = F[qrows].mean(0)
        sc = 32.0 / max(np.abs(F[qrows] - cref).max(), np.abs(B - cref).max())
        qa_c, qb_c = e4m3(sc * (A - cref)), e4m3(sc * (B - cref))
        dq["centred"] = ((qa_c[:, None, :] - qb_c[None, :, :]) ** 2).sum(-1)
        for mode, d in dq.items():
            d = np.where(np.isfinite(d64), d, np.inf)
            order = np.argsort(d, axis=1, kind="stable")
            for M in Ms:
                top = order[:, :M]
                hits[mode][M] += sum(len(set(t.tolist()) & set(r.tolist())) for t, r in zip(top, true))
        total += len(qs) * knn
    return {mode: {M: h / total for M, h in hm.items()} for mode, hm in hits.items()}, total


if __name__ == "__main__":
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from ironclust_gb300 import synth
    site = synth.make_workload("drift400k")
    res, n = ceiling(site["F"], synth.site_plan(site))
    print("drift400k, %d (query, true neighbour) pairs sampled" % n)
    for mode, r in res.items():
        print("  %-9s " % mode + "  ".join("M=%d: %.4f" % (M, v) for M, v in r.items()))
