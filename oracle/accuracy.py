"""Accuracy of a kNN / rho / delta result against the FP64 oracle
(TEST INFRASTRUCTURE ONLY: the tests, the smoke check and bench.py's
accuracy lines, outside their timed regions, use it as the checker).

The FP64 reference of a single-page site (every column of F a query):
  * kNN: the true k nearest candidates over the drift-linked runs, distance
    > 0, ties by (distance, index) -- ``exact_knn_f64``;
  * rho64 = 1 / d_knn in double;
  * delta64: the nearest candidate whose rho64 is strictly higher (the mask of
    search_delta_drift, matlab/search_delta_drift.cu:73-76, evaluated on the
    FP64 rho) -- ``exact_delta_f64`` -- times rho64 of the query (the
    ``delta .*= rho`` of delta_paged_site_, matlab/irc2.m:3720).

Nearest-higher-rho disagreements are counted, never filtered out.  A
disagreement whose candidate (the result's or the FP64 one) is ordered
differently against the query by the result's own rho and by rho64, while
the two rho64 values lie within FLIP_TOL of each other -- closer together
than an FP32 rho resolves -- is a "rho-order flip": any FP32 computation of
rho meets those, the exact FP32 form as much as a tensor-core one.  Every
other disagreement is an error.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

# Two rho64 values closer than this (relative) are below what an FP32 rho
# resolves (its rounding and the FP32 distance behind it: a few 1e-7).
FLIP_TOL = 1e-6


def fp64_reference(F, plan, knn):
    """dict(idx [n, knn] 1-based (0 = missing), d2 [n, knn] (NaN = missing),
    rho [n] (NaN where fewer than knn neighbours exist), nneigh [n] 1-based
    (0 = no higher-rho candidate), delta [n] (inf = none))."""
    if int(plan["q_base"]) != 0 or int(plan["n_out"]) != F.shape[0]:
        raise ValueError("fp64_reference: the plan must cover every column of F")
    idx, d2 = O.exact_knn_f64(F, plan, knn)
    with np.errstate(divide="ignore", invalid="ignore"):
        rho = 1.0 / np.sqrt(d2[:, knn - 1])
    nn, dd = O.exact_delta_f64(F, np.where(np.isnan(rho), -np.inf, rho), plan)
    with np.errstate(invalid="ignore"):
        delta = np.sqrt(dd) * rho
    return dict(idx=idx, d2=d2, rho=rho, nneigh=nn, delta=delta)


def knn_recall(got_idx, ref_idx, ref_d2):
    """Set overlap of the neighbours that exist (small chunks have fewer than k)."""
    got_idx = np.asarray(got_idx)
    nval = np.isfinite(ref_d2).sum(1)
    hits = 0
    for g, r, v in zip(got_idx, ref_idx, nval):
        if v:
            hits += len(set(g[:v].tolist()) & set(r[:v].tolist()))
    tot = int(nval.sum())
    return hits / tot if tot else 1.0


def compare(out, ref, queries=None):
    """Accuracy of `out` (numpy arrays miKnn [n, knn] 1-based, rho [n],
    delta [n], nneigh [n] 1-based, the query itself when none) against
    fp64_reference; `queries` restricts the check to a subset of rows."""
    n = ref["rho"].shape[0]
    sel = np.arange(n) if queries is None else np.asarray(queries)
    res = {"checked": int(sel.size)}
    res["recall_vs_fp64"] = knn_recall(out["miKnn"][sel], ref["idx"][sel], ref["d2"][sel])
    rho = np.asarray(out["rho"], np.float64)
    ok = np.isfinite(ref["rho"][sel])
    r64 = ref["rho"][sel][ok]
    rel = np.abs(rho[sel][ok] - r64) / r64
    res.update(rho_max_rel_err=float(rel.max()) if rel.size else 0.0,
               rho_mean_rel_err=float(rel.mean()) if rel.size else 0.0,
               rho_checked=int(ok.sum()))
    if "delta" in out and out["delta"] is not None:
        nn_got = np.asarray(out["nneigh"], np.int64)[sel]
        nn_ref = ref["nneigh"][sel].astype(np.int64)
        has_ref = nn_ref > 0
        has_got = nn_got != sel + 1
        d64 = ref["delta"][sel]
        dg = np.asarray(out["delta"], np.float64)[sel]
        both = has_ref & has_got & ok
        with np.errstate(divide="ignore", invalid="ignore"):
            drel = np.where(both, np.abs(dg - d64) / d64, 0.0)
        wrong = (nn_got != nn_ref) & has_ref | (has_ref != has_got)
        # rho-order flips: the result's FP32 rho and rho64 order a candidate
        # (the result's or the FP64 neighbour) differently against the query
        rq32, rq64 = rho[sel], ref["rho"][sel]

        def flipped(c):                          # c: 0-based candidate per row, -1 = none
            v = c >= 0
            cc = np.where(v, c, 0)
            with np.errstate(invalid="ignore"):
                o32 = rho[cc] > rq32
                o64 = ref["rho"][cc] > rq64
                close = np.abs(ref["rho"][cc] - rq64) <= FLIP_TOL * np.abs(rq64)
            return v & (o32 != o64) & close

        flip = wrong & (flipped(np.where(has_got, nn_got - 1, -1)) | flipped(np.where(has_ref, nn_ref - 1, -1)))
        err = wrong & ~flip
        ok_d = both & ~flip
        res.update(delta_max_rel_err=float(drel[ok_d].max()) if ok_d.any() else 0.0,
                   delta_mean_rel_err=float(drel[ok_d].mean()) if ok_d.any() else 0.0,
                   delta_max_rel_err_all=float(drel[both].max()) if both.any() else 0.0,
                   delta_checked=int(both.sum()), nneigh_wrong=int(wrong.sum()),
                   nneigh_rho_order_flips=int(flip.sum()), nneigh_errors=int(err.sum()),
                   delta_above_1e4=int((drel[ok_d] > 1e-4).sum()))
    return res


def stream_block_check(st, k, knn):
    """Accuracy of block k of a streamed pass (st: a stream.Streamer after
    run()) against FP64: kNN recall, rho and delta with the same rules as
    compare().  Block k's candidates and higher-rho neighbours lie in blocks
    k-1 .. k+1, so the FP64 kNN runs on those three blocks (their rho64), the
    FP64 delta on block k; everything is checked in the coordinates of that
    three-block window of the recording."""
    wl = st.wl
    nb, base, D = wl["n_blocks"], wl["block_base"], wl["n_dim"]
    ring = np.zeros((st.N_SLOTS * st.slot_rows, D), np.float32)
    for j in range(k - 2, k + 3):                # blocks k-1 .. k+1 read their own neighbours
        if 0 <= j < nb:
            a, z = int(base[j]), int(base[j + 1])
            ring[st._slot(j):st._slot(j) + (z - a)] = wl["F16"][a:z].numpy()
    js = [j for j in (k - 1, k, k + 1) if 0 <= j < nb]
    lo, hi = int(base[js[0]]), int(base[js[-1] + 1])
    W = hi - lo

    def to_window(ids):                          # 1-based ring rows of block k's plan -> window rows
        ids = np.asarray(ids, np.int64)
        out = np.zeros_like(ids)
        for j in js:
            r0, n = st._slot(j), int(base[j + 1] - base[j])
            sel = (ids > r0) & (ids <= r0 + n)
            out[sel] = ids[sel] - r0 + (int(base[j]) - lo)
        return out

    R = np.full(ring.shape[0], -np.inf)
    ref = dict(idx=np.zeros((W, knn), np.int64), d2=np.full((W, knn), np.nan), rho=np.full(W, np.nan),
               nneigh=np.zeros(W, np.int64), delta=np.full(W, np.inf))
    for j in js:
        idx, d2 = O.exact_knn_f64(ring, dict(st.plans[j].d), knn)
        with np.errstate(divide="ignore", invalid="ignore"):
            rho = 1.0 / np.sqrt(d2[:, knn - 1])
        n, w0 = int(base[j + 1] - base[j]), int(base[j]) - lo
        R[st._slot(j):st._slot(j) + n] = np.where(np.isnan(rho), -np.inf, rho)
        ref["rho"][w0:w0 + n] = rho
        if j == k:
            ref["idx"][w0:w0 + n] = to_window(idx)
            ref["d2"][w0:w0 + n] = d2
    nn, dd = O.exact_delta_f64(ring, R, dict(st.plans[k].d))
    a, z = int(base[k]), int(base[k + 1])
    q = np.arange(a - lo, z - lo)
    ref["nneigh"][q] = to_window(nn)
    with np.errstate(invalid="ignore"):
        ref["delta"][q] = np.sqrt(dd) * ref["rho"][q]
    out = dict(rho=st.out["rho"][lo:hi].numpy(), miKnn=np.zeros((W, knn), np.int64),
               nneigh=np.zeros(W, np.int64), delta=np.zeros(W, np.float32))
    out["miKnn"][q] = to_window(st.out["miKnn"][a:z].numpy())
    out["nneigh"][q] = to_window(st.out["nneigh"][a:z].numpy())
    out["delta"][q] = st.out["delta"][a:z].numpy()
    res = compare(out, ref, q)
    res.update(block=int(k), block_spikes=int(z - a))
    return res
