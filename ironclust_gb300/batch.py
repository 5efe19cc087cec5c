"""All probe sites as one batch: one feature matrix, one plan, one launch per kernel.

IronClust processes sites one by one in a parfor (matlab/irc2.m:3539-3561),
each site with its own feature dimension.  Here the sites of a probe are
stacked into one feature matrix, zero-padded to the largest dimension, and
their per-chunk launch plans are concatenated with row offsets.  A padded
feature is 0 for every spike of its site, so it adds exactly 0 to each fused
accumulate: every distance, and so every result, equals the per-site one
bit for bit.  Candidate runs never cross sites, so the batch is a plan like
any other and runs through irc_plan_create / irc_site_knn / irc_site_delta
in one launch per kernel; the tensor-core kernel packs the small chunks of
many sites into shared CTAs.
"""
from __future__ import annotations

import numpy as np

from .drift import build_plan


class SiteBatch:
    """sites: iterable of dict(F [n, D] float32, viDrift [n], mlDrift [nDrift x nDrift])."""

    def __init__(self, sites):
        sites = list(sites)
        Fs = [s["F"] for s in sites]
        plans = [build_plan(s["viDrift"], np.ones(s["F"].shape[0], bool), s["mlDrift"]) for s in sites]
        self._stack(Fs, plans)

    def subset(self, idx):
        """The batch of sites idx (in that order), e.g. one rank's share.  It
        keeps this batch's padded width, so every kernel sees the same
        feature layout and its results equal this batch's rows bit for bit."""
        out = SiteBatch.__new__(SiteBatch)
        out._stack([self.F[self.site_slice(i), :int(self.dims[i])] for i in idx], [self.site_plans[i] for i in idx],
                   width=self.F.shape[1])
        return out

    def _stack(self, Fs, plans, width=None):
        self.n_sites = len(Fs)
        self.dims = np.array([f.shape[1] for f in Fs], np.int32)
        self.sizes = np.array([f.shape[0] for f in Fs], np.int64)
        self.bases = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        n, dmax = int(self.bases[-1]), int(width or self.dims.max())
        self.F = np.zeros((n, dmax), np.float32)
        q0, nq, rs, rn, roff, site_of_chunk = [], [], [], [], [0], []
        self.site_plans = []
        for i, (f, p) in enumerate(zip(Fs, plans)):
            b = int(self.bases[i])
            self.F[b:b + f.shape[0], :f.shape[1]] = f
            self.site_plans.append(p)
            q0.append(p["q0"] + b)
            nq.append(p["nq"])
            rs.append(p["rs"] + b)
            rn.append(p["rn"])
            roff.extend((p["roff"][1:] + roff[-1]).tolist())
            site_of_chunk.append(np.full(len(p["q0"]), i, np.int32))
        i32 = lambda parts: np.concatenate(parts).astype(np.int32)
        self.plan = dict(q0=i32(q0), nq=i32(nq), roff=np.asarray(roff, np.int32), rs=i32(rs), rn=i32(rn),
                         q_base=0, n_out=n, n_f=n)
        self.site_of_chunk = np.concatenate(site_of_chunk)

    def site_slice(self, i):
        return slice(int(self.bases[i]), int(self.bases[i + 1]))

    def split_knn(self, miKnn, i):
        """kNN rows of site i with indices local to that site (1-based)."""
        return np.asarray(miKnn)[self.site_slice(i)] - int(self.bases[i])

    def make_plan(self):
        """irc.Plan of the batch with its site widths set
        (irc_plan_set_site_dims): the tensor-core re-rank skips each site's
        padded features."""
        from . import irc
        return irc.Plan(self.plan).set_site_dims(self.bases, self.dims)

    def c_plan(self):
        """The batch plan built by the library from the per-site plans
        (irc_batch_plan_create), the route of a C or MATLAB host."""
        import ctypes as C

        from . import irc
        from ._lib import check, lib
        cat = lambda k: np.ascontiguousarray(np.concatenate([p[k] for p in self.site_plans]), np.int32)
        nch = np.array([len(p["q0"]) for p in self.site_plans], np.int32)
        arrs = [nch, np.ascontiguousarray(self.bases, np.int64), cat("q0"), cat("nq"), cat("roff"), cat("rs"),
                cat("rn")]
        h = C.c_void_p()
        check(lib().irc_batch_plan_create(C.byref(h), self.n_sites, *[a.ctypes.data_as(C.c_void_p) for a in arrs]),
              "irc_batch_plan_create")
        return irc.Plan.from_handle(h, self.plan).set_site_dims(self.bases, self.dims)

    def stack_device(self, F_sites):
        """The stacked feature matrix from per-site device tensors
        (irc_batch_stack): [n, max D] float32, zero-padded."""
        import ctypes as C

        import torch

        from ._lib import check, lib
        dev = F_sites[0].device
        n, dmax = int(self.bases[-1]), int(self.F.shape[1])
        out = torch.empty((n, dmax), dtype=torch.float32, device=dev)
        ptrs = (C.c_void_p * self.n_sites)(*[t.data_ptr() for t in F_sites])
        nc = np.ascontiguousarray(self.dims, np.int32)
        rb = np.ascontiguousarray(self.bases, np.int64)
        check(lib().irc_batch_stack(C.c_void_p(out.data_ptr()), dmax, C.cast(ptrs, C.c_void_p),
                                    nc.ctypes.data_as(C.c_void_p), rb.ctypes.data_as(C.c_void_p), self.n_sites,
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)), "irc_batch_stack")
        return out

