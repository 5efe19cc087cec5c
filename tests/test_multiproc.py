"""Site sharding over ranks (gloo, world size 2): every rank takes its LPT
share of a batch of sites (shard.batch_share), computes kNN, rho and delta of
that sub-batch with no data exchange, and rank 0 merges the shares by global
spike id (shard.gather_merge).  The merged outputs equal a single-process run
over the whole batch bit for bit.

On CPU the ranks run the oracle (the reference's CPU path, knn_cpu_ +
delta_cpu_ restated); with a GPU both ranks run the
library on cuda:0 (independent processes, none waits on the other's kernels).
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from ironclust_gb300 import shard, synth
from ironclust_gb300.batch import SiteBatch

KNN = 10
CPU_SPECS = [(900, 6, 3, 3), (400, 8, 3, 2), (1200, 6, 4, 4), (300, 5, 2, 1), (700, 7, 3, 2), (500, 6, 3, 3)]
GPU_SPECS = [(9000, 33, 12, 6), (3000, 24, 8, 4), (12000, 18, 16, 8), (700, 33, 4, 2), (5000, 24, 10, 5),
             (2500, 18, 6, 3), (8000, 33, 14, 6)]


def make_batch(specs):
    return SiteBatch(synth.make_site(n, d, k, c, seed=500 + i) for i, (n, d, k, c) in enumerate(specs))


def compute(b, kind):
    """kNN + rho + delta of a (sub-)batch, host arrays."""
    if kind == "oracle":
        from oracle import oracle as O
        vr, mi = O.site_knn_cpu(b.F, b.plan, KNN)
        rho = (np.float32(1) / vr).astype(np.float32)
        delta, nn = O.site_delta_cpu(b.F, rho, b.plan)
        return dict(vrKnn=vr, miKnn=mi, rho=rho, delta=delta, nneigh=nn)
    from ironclust_gb300 import irc
    P = irc.Plan(b.plan)
    try:
        o = irc.knn_rho_delta_site(P, torch.from_numpy(b.F).cuda(), knn=KNN, mode=kind)
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in o.items() if v is not None}
    finally:
        P.close()


def _worker(rank, world, port, q, specs, kind):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = make_batch(specs)
        idx, sub = shard.batch_share(b, rank, world)
        merged = shard.gather_merge(b, idx, compute(sub, kind), rank, world)
        if rank == 0:
            q.put((shard.assign_sites(shard.batch_costs(b), world), merged))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_two_ranks(specs, kind):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, specs, kind)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = q.get(timeout=300)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    return got


def assert_bitwise_equal(merged, whole):
    assert sorted(merged) == sorted(whole)
    for k, v in whole.items():
        a, b = np.asarray(merged[k]), np.asarray(v)
        assert a.dtype == b.dtype and a.shape == b.shape, k
        assert np.array_equal(a.view(np.int32) if a.dtype == np.float32 else a,
                              b.view(np.int32) if b.dtype == np.float32 else b), k


def test_two_ranks_oracle_shares_equal_one_process():
    (assignment, merged) = run_two_ranks(CPU_SPECS, "oracle")
    assert sorted(i for part in assignment for i in part) == list(range(len(CPU_SPECS)))
    assert all(part for part in assignment)                   # both ranks had work
    assert_bitwise_equal(merged, compute(make_batch(CPU_SPECS), "oracle"))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["ref", "exact", "bf16"])
def test_two_ranks_library_shares_equal_one_process(gpu, mode):
    assignment, merged = run_two_ranks(GPU_SPECS, mode)
    assert all(part for part in assignment)
    assert_bitwise_equal(merged, compute(make_batch(GPU_SPECS), mode))


def test_merge_moves_ids_by_the_site_offset():
    b = make_batch(CPU_SPECS[:3])
    whole = {"nneigh": np.concatenate([np.arange(1, n + 1, dtype=np.int32) + int(b.bases[i])
                                       for i, n in enumerate(b.sizes)]),
             "rho": np.arange(int(b.bases[-1]), dtype=np.float32)}
    shares = []
    for idx in ([2, 0], [1]):
        sub = b.subset(idx)
        out = {"nneigh": np.concatenate([np.arange(1, int(b.sizes[s]) + 1, dtype=np.int32) + int(sub.bases[j])
                                         for j, s in enumerate(idx)]),
               "rho": np.concatenate([whole["rho"][b.site_slice(s)] for s in idx])}
        shares.append((idx, out))
    assert_bitwise_equal(shard.merge_shares(b, shares), whole)
    with pytest.raises(ValueError):
        shard.merge_shares(b, shares[:1])                     # site 1 in no share


def test_subset_keeps_sites_and_width():
    b = make_batch(CPU_SPECS)
    idx, sub = shard.batch_share(b, 1, 2)
    assert sub.F.shape[1] == b.F.shape[1]
    for j, s in enumerate(idx):
        assert np.array_equal(sub.F[sub.site_slice(j)], b.F[b.site_slice(s)])
        for k in ("q0", "nq", "rs", "rn", "roff"):
            assert np.array_equal(sub.site_plans[j][k], b.site_plans[s][k])


def test_assignment_is_balanced_for_the_probe_workload():
    specs = synth.probe_site_specs(n_sites=384)
    costs = [s["n_spk"] ** 2 // 80 * s["n_dim"] for s in specs]
    for w in (2, 4, 8):
        a = shard.assign_sites(costs, w)
        assert shard.imbalance(costs, a) < 1.10
