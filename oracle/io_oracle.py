"""numpy restatement of the on-disk formats around the path: TEST
INFRASTRUCTURE ONLY (writes reference-format fixtures and reads them the way
the MATLAB code does; only tests/ import it).

* ``write_fet_files``   detect_paged_save_ + save_paged_fet_site_,
                        matlab/irc2.m:4582-4618: one file per load, site after
                        site, each spike a [nPc x nSites_spk] single record
* ``load_fet_site``     load_fet_site_, matlab/irc2.m:4039-4135
* ``knn_rows``          rho_paged_site_'s kNN rows, matlab/irc2.m:3670-3676
* ``sort_bytes``        struct_save_bin_ of rho, delta, nneigh, ordrho,
                        matlab/irc2.m:356-391, :1733-1750
"""
from __future__ import annotations

import os

import numpy as np


def write_fet_files(prefix, tr_by_load, site_by_load, n_sites, tag="_fet_"):
    """tr_by_load[l]: [n_l, nSites_spk, nPc] float32 (spike-major; MATLAB
    trPc_spk(:,:,i) is tr[i].T); site_by_load[l]: 0-based primary site of each
    spike of load l.  Spike ids are global, 1-based, in load order.  Returns
    (files, ccviSpk_site_load)."""
    files, cc = [], []
    first = 1
    for l, (tr, site) in enumerate(zip(tr_by_load, site_by_load)):
        path = "%s%s%d.irc" % (prefix, tag, l + 1)
        ids = np.arange(first, first + len(site), dtype=np.int64)
        per_site = []
        with open(path, "wb") as f:
            for s in range(n_sites):
                k = np.flatnonzero(site == s)             # vi2cell_: ascending
                per_site.append(ids[k])
                # MATLAB [nPc x nSites_spk x n] column-major = spike-major
                # records of nSites_spk x nPc (PC fastest)
                f.write(np.ascontiguousarray(tr[k], np.float32).tobytes())
        files.append(path)
        cc.append(per_site)
        first += len(site)
    return files, cc


def load_fet_site(files, cc, iSite, viSpk, n_pc, n_sites_spk, mlPc=None):
    """MATLAB's load_fet_site_ on those files: [nOut, nC] float32 (row =
    MATLAB column), columns load by load, within a load in viSpk order."""
    rec = n_pc * n_sites_spk
    lin = np.arange(rec) if mlPc is None else np.flatnonzero(np.asarray(mlPc, bool).T.reshape(-1))
    out = []
    for path, load in zip(files, cc):
        n_before = sum(len(x) for x in load[:iSite])
        site_ids = load[iSite]
        if not len(site_ids):
            continue
        data = np.fromfile(path, np.float32, count=len(site_ids) * rec, offset=n_before * rec * 4)
        data = data.reshape(len(site_ids), rec)
        if viSpk is None:
            pick = np.arange(len(site_ids))
        else:
            pos = {int(v): i for i, v in enumerate(site_ids)}
            pick = np.array([pos[int(v)] for v in viSpk if int(v) in pos], np.int64)
        out.append(data[pick][:, lin])
    return np.concatenate(out) if out else np.zeros((0, len(lin)), np.float32)


def knn_rows(miKnn, viSpk_out, knn):
    """int64 [n, knn] rows (MATLAB [knn x n]): global ids of the 1-based
    positions, padded by repeating the last row."""
    mi = np.asarray(viSpk_out, np.int64)[np.asarray(miKnn, np.int64) - 1]
    if mi.shape[1] < knn:
        mi = np.concatenate([mi, np.repeat(mi[:, -1:], knn - mi.shape[1], axis=1)], axis=1)
    return mi


def sort_bytes(rho, delta, nneigh, ordrho):
    return (np.asarray(rho, np.float32).tobytes() + np.asarray(delta, np.float32).tobytes()
            + np.asarray(nneigh, np.int64).tobytes() + np.asarray(ordrho, np.float64).tobytes())
