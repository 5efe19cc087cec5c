"""Multi-day scale on one GPU: a long recording streamed from pinned host
memory, page by page, through the tensor-core path.

Shape (the reference's largest runs scaled up): 100M spikes across 384
sites, D = 33 features stored as FP16 in pinned host memory, 10,000 drift
chunks with a random-walk plus slow linear drift, every chunk linked to its
15 most similar chunks within +-64 (one linkage for the recording, as
calc_drift_ computes one from all spikes), knn = 30.

The recording is paged as sort_page_ pages it (plan_sort_page_,
matlab/irc2.m:3914-3946): blocks of 128 drift chunks are the query ranges,
and a block's linked chunks lie in the blocks before and after it.  The host
buffer is block-major (block k = every site's spikes in chunks 128k ..
128k+127, site after site), so a block streams as one contiguous copy.  The
device keeps a ring of five block slots: kNN of block k+1 and delta of block
k read blocks k-1 .. k+2 while block k+3 is copied in (and widened from FP16
to FP32) on its own stream; a third stream returns finished blocks' results
(rho, delta, nneigh, kNN) to pinned host memory.  One plan per block
addresses its rows in ring coordinates; all block plans share one
tensor-core working buffer.  A block spans a bounded stretch of drift, so
the centring of the tensor-core operands (on the plan's own queries) keeps
them small however far the recording drifts.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import irc
from ._lib import check, lib
from .drift import chunk_limits


def _p(t):
    return C.c_void_p(t.data_ptr())


def band_members(offs, n_link=15, band=64):
    """Column j: the n_link chunks nearest chunk j (Euclidean distance of the
    drift offsets) within calc_drift_'s +-band mask (one interval of rows),
    self first.  [n_link, n_chunks] int64, ascending chunk id per column."""
    n = offs.shape[0]
    q = band
    out = np.empty((n_link, n), np.int64)
    for j in range(n):
        if n <= 4 * q:
            lo, hi = 0, n - 1
        elif j < q:
            lo, hi = 0, 2 * q
        elif j >= n - q:
            lo, hi = n - 2 * q - 1, n - 1
        else:
            lo, hi = j - q, j + q
        d = ((offs[lo:hi + 1] - offs[j]) ** 2).sum(1)
        d[j - lo] = -1.0                               # self first, exactly
        out[:, j] = np.sort(lo + np.argpartition(d, n_link - 1)[:n_link])
    return out


def make_workload(n_sites=384, total=100_000_000, n_chunks=10_000, n_dim=33, seed=1004, drift_sd=0.3,
                  drift_slope=0.01, noise_frac=0.05, n_link=15, band=64, block_chunks=128, pin=True):
    """Synthetic recording of the multi-day shape in block-major order.

    Returns dict(F16 [N, D] float16 (pinned torch tensor, block-major), lims
    [n_sites, n_chunks+1] per-site chunk limits (site-local spike order),
    seg [n_blocks, n_sites] row of each site's segment in the host buffer,
    block_base [n_blocks+1], members, offs, ...)."""
    rng = np.random.default_rng(seed)
    n = np.clip(np.exp(rng.normal(np.log(20000), 1.0, n_sites)), 500, 2_000_000)
    sizes = np.maximum((n * total / n.sum()).astype(np.int64), 500)
    N = int(sizes.sum())
    steps = rng.normal(0.0, drift_sd, (n_chunks, n_dim))
    steps[0] = 0.0
    offs = np.cumsum(steps, axis=0) + drift_slope * np.arange(n_chunks)[:, None]
    members = band_members(offs, n_link, band)
    nb = (n_chunks + block_chunks - 1) // block_chunks
    bchunk = np.minimum(np.arange(nb + 1) * block_chunks, n_chunks)        # first chunk of each block
    lims = np.stack([chunk_limits(int(ns), n_chunks) for ns in sizes])    # [S, n_chunks+1]
    seg_cnt = (lims[:, bchunk[1:]] - lims[:, bchunk[:-1]]).T              # [nb, S]
    flat = np.concatenate([[0], np.cumsum(seg_cnt.reshape(-1))])
    seg = flat[:-1].reshape(nb, n_sites)
    block_base = flat[np.arange(nb + 1) * n_sites]
    F16 = torch.empty((N, n_dim), dtype=torch.float16, pin_memory=pin)
    view = F16.numpy()
    for s in range(n_sites):
        ns = int(sizes[s])
        r = np.random.default_rng(seed * 1000 + s)
        k = int(r.integers(12, 41))
        centres = r.normal(0.0, 10.0, (k, n_dim)).astype(np.float32)
        sds = r.uniform(0.5, 2.0, (k, n_dim)).astype(np.float32)
        w = r.dirichlet(np.ones(k))
        chunk = np.repeat(np.arange(n_chunks), np.diff(lims[s]))
        lab = r.choice(k, size=ns, p=w)
        F = centres[lab] + offs[chunk].astype(np.float32) + sds[lab] * r.standard_normal((ns, n_dim), np.float32)
        n_noise = int(round(noise_frac * ns))
        if n_noise:
            lo, hi = F.min(0), F.max(0)
            ii = r.choice(ns, size=n_noise, replace=False)
            F[ii] = r.uniform(lo, hi, (n_noise, n_dim)).astype(np.float32)
        F = F.astype(np.float16)
        for kb in range(nb):
            a, z = int(lims[s, bchunk[kb]]), int(lims[s, bchunk[kb + 1]])
            if z > a:
                view[seg[kb, s]:seg[kb, s] + (z - a)] = F[a:z]
    return dict(F16=F16, sizes=sizes, lims=lims, seg=seg, block_base=block_base, bchunk=bchunk, members=members,
                offs=offs, n_dim=n_dim, n_chunks=n_chunks, n_blocks=nb, block_chunks=block_chunks)


def block_plan(wl, k, slot_rows, n_slots=4):
    """Plan of query block k with rows in ring coordinates (block j in slot
    j % n_slots, slot_rows rows per slot)."""
    lims, seg, base, Bc = wl["lims"], wl["seg"], wl["block_base"], wl["block_chunks"]
    S = lims.shape[0]
    c0, c1 = int(wl["bchunk"][k]), int(wl["bchunk"][k + 1])
    cs = np.arange(c0, c1)

    def rows(sites, chunks):                       # ring row of the first spike of (site, chunk)
        kb = chunks // Bc
        return ((kb % n_slots) * slot_rows + (seg[kb, sites] - base[kb])
                + (lims[sites, chunks] - lims[sites, kb * Bc]))

    s_idx = np.repeat(np.arange(S), len(cs))       # (site, chunk) pairs, site-major
    c_idx = np.tile(cs, S)
    qcnt = lims[s_idx, c_idx + 1] - lims[s_idx, c_idx]
    qk = qcnt > 0
    s_q, c_q = s_idx[qk], c_idx[qk]
    mem = wl["members"][:, c_q]                    # [L, nQ] linked chunks, ascending
    s_b = np.broadcast_to(s_q, mem.shape)
    bcnt = lims[s_b, mem + 1] - lims[s_b, mem]
    keep = bcnt > 0
    per = keep.sum(0)
    mem_t, s_bt, keep_t, bcnt_t = mem.T, s_b.T, keep.T, bcnt.T
    i32 = lambda v: np.asarray(v, np.int32)
    n_out = int(base[k + 1] - base[k])
    return dict(q0=i32(rows(s_q, c_q)), nq=i32(qcnt[qk]), roff=i32(np.concatenate([[0], np.cumsum(per)])),
                rs=i32(rows(s_bt[keep_t], mem_t[keep_t])), rn=i32(bcnt_t[keep_t]),
                q_base=(k % n_slots) * slot_rows, n_out=n_out, n_f=n_slots * slot_rows)


class Streamer:
    """The page-streaming pipeline (plans and device buffers made once,
    outside any timed region).

    Order on the compute stream: kNN(0), then for every block k kNN(k+1)
    followed by delta(k) -- delta needs the rho of blocks k-1 .. k+1, so kNN
    runs one block ahead.  The ring therefore holds five blocks (k-1 .. k+2
    read by kNN(k+1) and delta(k), k+3 copied in meanwhile); rho lives in a
    ring of the same shape, and the per-block outputs (kNN lists, delta,
    nneigh) rotate through three buffers so the copy back of block k overlaps
    kNN(k+2) and delta(k+1)."""

    N_SLOTS = 5
    N_OUT = 3

    def __init__(self, wl, knn=30, mode="bf16", device="cuda"):
        self.wl, self.knn, self.mode, self.dev = wl, knn, mode, torch.device(device)
        nb = wl["n_blocks"]
        base = wl["block_base"]
        self.slot_rows = int(np.max(np.diff(base)))
        self.slot_rows += (-self.slot_rows) % 4                         # 16-byte aligned slots
        D = wl["n_dim"]
        R = self.N_SLOTS * self.slot_rows
        self.f16 = torch.zeros((R, D), dtype=torch.float16, device=self.dev)
        self.f32 = torch.zeros((R, D), dtype=torch.float32, device=self.dev)
        self.rho = torch.zeros(R, dtype=torch.float32, device=self.dev)
        self.plans = [irc.Plan(block_plan(wl, k, self.slot_rows, self.N_SLOTS)) for k in range(nb)]
        tc_bytes = max(lib().irc_plan_tc_bytes(P.h, D) for P in self.plans)   # n_out differs per block
        self.tc = torch.empty(tc_bytes, dtype=torch.uint8, device=self.dev)
        for P in self.plans:
            check(lib().irc_plan_set_tc_buffer(P.h, _p(self.tc), C.c_size_t(tc_bytes)), "irc_plan_set_tc_buffer")
        m = self.slot_rows
        self.vrKnn = torch.empty(m, dtype=torch.float32, device=self.dev)
        self.buf = [dict(mi=torch.empty((m, knn), dtype=torch.int32, device=self.dev),
                         d2=torch.empty((m, knn), dtype=torch.float32, device=self.dev),
                         delta=torch.empty(m, dtype=torch.float32, device=self.dev),
                         nneigh=torch.empty(m, dtype=torch.int32, device=self.dev)) for _ in range(self.N_OUT)]
        N = int(base[-1])
        pin = torch.cuda.is_available()
        self.out = dict(rho=torch.empty(N, dtype=torch.float32, pin_memory=pin),
                        delta=torch.empty(N, dtype=torch.float32, pin_memory=pin),
                        nneigh=torch.empty(N, dtype=torch.int32, pin_memory=pin),
                        miKnn=torch.empty((N, knn), dtype=torch.int32, pin_memory=pin))
        self.s_in, self.s_run, self.s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()

    def _slot(self, j):
        return (j % self.N_SLOTS) * self.slot_rows

    def _copy_in(self, j):
        """Block j into its slot, widened to FP32 (stream s_in), once delta of
        the slot's previous block (j - 5, read by delta(j - 4)) is done."""
        base = self.wl["block_base"]
        a, z = int(base[j]), int(base[j + 1])
        r0 = self._slot(j)
        D = self.wl["n_dim"]
        with torch.cuda.stream(self.s_in):
            if j - 4 >= 0:
                self.s_in.wait_event(self.ev_delta[j - 4])
            self.f16[r0:r0 + (z - a)].copy_(self.wl["F16"][a:z], non_blocking=True)
            check(lib().irc_f16_to_f32(_p(self.f32[r0:]), _p(self.f16[r0:]), C.c_int64((z - a) * D),
                                       C.c_void_p(self.s_in.cuda_stream)), "irc_f16_to_f32")
            self.ev_in[j].record(self.s_in)

    def _knn(self, k):
        """kNN + rho of block k (rho into its ring slot); needs blocks k-1 .. k+1."""
        nb = self.wl["n_blocks"]
        B = self.buf[k % self.N_OUT]
        D = self.wl["n_dim"]
        with torch.cuda.stream(self.s_run):
            self.s_run.wait_event(self.ev_in[min(k + 1, nb - 1)])
            if k - self.N_OUT >= 0:
                self.s_run.wait_event(self.ev_out[k - self.N_OUT])   # this output buffer went back
            check(lib().irc_site_knn(self.plans[k].h, _p(self.f32), D, self.knn, 1024, irc._mode(self.mode),
                                     _p(self.vrKnn), _p(self.rho[self._slot(k):]), _p(B["mi"]), _p(B["d2"]),
                                     C.c_void_p(self.s_run.cuda_stream)), "irc_site_knn")

    def _delta(self, k):
        B = self.buf[k % self.N_OUT]
        D = self.wl["n_dim"]
        with torch.cuda.stream(self.s_run):
            check(lib().irc_site_delta(self.plans[k].h, _p(self.f32), D, _p(self.rho), 512, irc._mode(self.mode),
                                       self.knn, _p(B["mi"]), _p(B["d2"]), _p(B["delta"]), _p(B["nneigh"]),
                                       C.c_void_p(self.s_run.cuda_stream)), "irc_site_delta")
            self.ev_delta[k].record(self.s_run)

    def _copy_out(self, k):
        base = self.wl["block_base"]
        a, z = int(base[k]), int(base[k + 1])
        n = z - a
        B = self.buf[k % self.N_OUT]
        r0 = self._slot(k)
        with torch.cuda.stream(self.s_out):
            self.s_out.wait_event(self.ev_delta[k])
            self.out["rho"][a:z].copy_(self.rho[r0:r0 + n], non_blocking=True)
            self.out["delta"][a:z].copy_(B["delta"][:n], non_blocking=True)
            self.out["nneigh"][a:z].copy_(B["nneigh"][:n], non_blocking=True)
            self.out["miKnn"][a:z].copy_(B["mi"][:n], non_blocking=True)
            self.ev_out[k].record(self.s_out)

    def run(self):
        """One pass over the recording; returns the wall time (ms, CUDA events
        from the first copy in to the last copy out).  Neighbour indices in
        out["miKnn"] / out["nneigh"] are 1-based ring rows of the block's own
        computation (to_global maps them to recording rows)."""
        nb = self.wl["n_blocks"]
        self.ev_in = [torch.cuda.Event() for _ in range(nb)]
        self.ev_delta = [torch.cuda.Event() for _ in range(nb)]
        self.ev_out = [torch.cuda.Event() for _ in range(nb)]
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(self.s_in)
        for j in range(min(3, nb)):
            self._copy_in(j)
        self._knn(0)
        for k in range(nb):
            if k + 3 < nb:
                self._copy_in(k + 3)
            if k + 1 < nb:
                self._knn(k + 1)
            self._delta(k)
            self._copy_out(k)
        self.s_in.wait_stream(self.s_out)
        self.s_in.wait_stream(self.s_run)
        t1.record(self.s_in)
        t1.synchronize()
        return t0.elapsed_time(t1)

    def to_global(self, k, idx):
        """1-based ring rows of block k's computation -> 1-based rows of the
        recording (0 stays 0)."""
        idx = np.asarray(idx, np.int64)
        base = self.wl["block_base"]
        out = np.zeros_like(idx)
        for j in (k - 1, k, k + 1):
            if 0 <= j < self.wl["n_blocks"]:
                r0 = self._slot(j)
                sel = (idx > r0) & (idx <= r0 + int(base[j + 1] - base[j]))
                out[sel] = idx[sel] - r0 + int(base[j])
        return out

    def ring_rows(self, k):
        """Host copy of the ring as block k's computation sees it (blocks
        k-1 .. k+1 in their slots, other rows zero): for checks."""
        base = self.wl["block_base"]
        F = np.zeros((self.N_SLOTS * self.slot_rows, self.wl["n_dim"]), np.float32)
        for j in (k - 1, k, k + 1):
            if 0 <= j < self.wl["n_blocks"]:
                r0 = self._slot(j)
                F[r0:r0 + int(base[j + 1] - base[j])] = self.wl["F16"][int(base[j]):int(base[j + 1])].numpy()
        return F

    def block_rows(self, k):
        base = self.wl["block_base"]
        return int(base[k]), int(base[k + 1])

    def bytes_per_pass(self):
        N = int(self.wl["block_base"][-1])
        return N * self.wl["n_dim"] * 2, N * (4 + 4 + 4 + 4 * self.knn)

    def close(self):
        for P in self.plans:
            P.close()
