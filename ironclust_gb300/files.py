"""The on-disk formats around the path, read into and written from device
memory through libircgb300 (irc_fet_load_site, irc_knn_save_site,
irc_sort_save / irc_sort_load).

The spike bookkeeping of load_fet_site_ (matlab/irc2.m:4039-4135) stays on
the host -- which records of which load a site's wanted spikes are -- and
the library streams the records to the device and gathers the features.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import check, lib


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def fet_selection(ccviSpk_site_load, iSite, viSpk=None):
    """Host side of load_fet_site_: per load, the records of the sites before
    iSite and of iSite, and for the wanted spikes viSpk (global ids, in the
    order MATLAB returns them: load by load, within a load in viSpk order)
    their 0-based indices into the site's records concatenated over loads.
    ccviSpk_site_load[l][s]: global spike ids of site s in load l (0-based
    site index here).  viSpk None = every spike of the site.  Returns
    (before, counts, viSel or None, spikes)."""
    before = np.array([sum(len(x) for x in load[:iSite]) for load in ccviSpk_site_load], np.int64)
    counts = np.array([len(load[iSite]) for load in ccviSpk_site_load], np.int64)
    if viSpk is None:
        spikes = np.concatenate([np.asarray(load[iSite], np.int64) for load in ccviSpk_site_load]) \
            if counts.sum() else np.zeros(0, np.int64)
        return before, counts, None, spikes
    viSpk = np.asarray(viSpk, np.int64)
    sel, spk = [], []
    base = 0
    for load, cnt in zip(ccviSpk_site_load, counts):
        site = np.asarray(load[iSite], np.int64)         # ascending (vi2cell_)
        if cnt:
            i = np.searchsorted(site, viSpk)
            hit = (i < cnt) & (site[np.minimum(i, cnt - 1)] == viSpk)
            sel.append(base + i[hit])
            spk.append(viSpk[hit])
        base += int(cnt)
    cat = lambda x: np.concatenate(x) if x else np.zeros(0, np.int64)
    return before, counts, cat(sel).astype(np.int64), cat(spk).astype(np.int64)


def fet_load_site(files, before, counts, nPc, nSitesSpk, mlPc=None, viSel=None, device="cuda"):
    """irc_fet_load_site: F as a [nOut, nC] CUDA tensor (== MATLAB [nC x nOut])."""
    n_rec = int(np.sum(counts))
    n_out = n_rec if viSel is None else len(viSel)
    ml = None if mlPc is None else np.ascontiguousarray(np.asarray(mlPc, bool).T.reshape(-1), np.uint8)
    n_c = nPc * nSitesSpk if ml is None else int(ml.sum())
    F = torch.empty((max(n_out, 1), max(n_c, 1)), dtype=torch.float32, device=device)
    sel = None if viSel is None else torch.as_tensor(np.asarray(viSel, np.int64), device=device)
    arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
    b = np.ascontiguousarray(before, np.int64)
    c = np.ascontiguousarray(counts, np.int64)
    nc = C.c_int(0)
    check(lib().irc_fet_load_site(_p(F), C.byref(nc), C.cast(arr, C.c_void_p), len(files),
                                  b.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p), nPc, nSitesSpk,
                                  None if ml is None else ml.ctypes.data_as(C.c_void_p), _p(sel),
                                  C.c_int64(n_out), _stream()), "irc_fet_load_site")
    return F[:n_out, :nc.value]


def knn_save_site(path, miKnn, viSpk, knn, append=False):
    """irc_knn_save_site: miKnn [n, knnIn] int32 1-based positions (CUDA),
    viSpk [nF] int64 global ids (CUDA) -> int64 [knn x n] appended/written."""
    miKnn = miKnn.to(torch.int32).contiguous()
    viSpk = viSpk.to(torch.int64).contiguous()
    n, knn_in = miKnn.shape
    check(lib().irc_knn_save_site(str(path).encode(), int(bool(append)), _p(miKnn), knn_in, knn, C.c_int64(n),
                                  _p(viSpk), C.c_int64(viSpk.numel()), _stream()), "irc_knn_save_site")


def sort_save(path, rho, delta, nneigh, ordrho):
    """irc_sort_save: rho, delta (float32), nneigh, ordrho (int64) CUDA tensors."""
    rho, delta = rho.float().contiguous(), delta.float().contiguous()
    nneigh, ordrho = nneigh.to(torch.int64).contiguous(), ordrho.to(torch.int64).contiguous()
    check(lib().irc_sort_save(str(path).encode(), _p(rho), _p(delta), _p(nneigh), _p(ordrho),
                              C.c_int64(rho.numel()), _stream()), "irc_sort_save")


def sort_load(path, n_spk, device="cuda"):
    """irc_sort_load: (rho, delta, nneigh, ordrho) CUDA tensors."""
    rho = torch.empty(n_spk, dtype=torch.float32, device=device)
    delta = torch.empty(n_spk, dtype=torch.float32, device=device)
    nneigh = torch.empty(n_spk, dtype=torch.int64, device=device)
    ordrho = torch.empty(n_spk, dtype=torch.int64, device=device)
    check(lib().irc_sort_load(str(path).encode(), _p(rho), _p(delta), _p(nneigh), _p(ordrho), C.c_int64(n_spk),
                              _stream()), "irc_sort_load")
    return rho, delta, nneigh, ordrho
