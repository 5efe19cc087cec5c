"""Site sharding over ranks on CPU (gloo, world size 2): every rank computes
its LPT share of the sites with no data exchange, the gathered results cover
every site exactly once and equal a single-process run."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from ironclust_gb300 import shard, synth
from ironclust_gb300.drift import plan_pairs

SPECS = [(900, 6, 3, 3), (400, 8, 3, 2), (1200, 6, 4, 4), (300, 5, 2, 1), (700, 7, 3, 2), (500, 6, 3, 3)]


def _site_result(i):
    from oracle import oracle as O
    n, d, k, c = SPECS[i]
    s = synth.make_site(n, d, k, c, seed=500 + i)
    plan = synth.site_plan(s)
    idx, d2 = O.exact_knn_f32(s["F"], plan, 10)
    return i, idx, d2


def _costs():
    out = []
    for i, (n, d, k, c) in enumerate(SPECS):
        s = synth.make_site(n, d, k, c, seed=500 + i)
        out.append(shard.site_cost(plan_pairs(synth.site_plan(s)), d))
    return out


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.rank_sites(_costs(), rank, world)
    res = [_site_result(i) for i in mine]
    gathered = [None] * world
    dist.all_gather_object(gathered, res)
    if rank == 0:
        q.put([r for part in gathered for r in part])
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_cover_every_site_once_and_match_one_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        results = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    got = {i: (idx, d2) for i, idx, d2 in results}
    assert sorted(got) == list(range(len(SPECS)))
    for i in range(len(SPECS)):
        _, idx, d2 = _site_result(i)
        assert np.array_equal(got[i][0], idx) and np.array_equal(got[i][1].view(np.int32), d2.view(np.int32))


def test_assignment_is_balanced_for_the_probe_workload():
    specs = synth.probe_site_specs(n_sites=384)
    costs = [s["n_spk"] ** 2 // 80 * s["n_dim"] for s in specs]
    for w in (2, 4, 8):
        a = shard.assign_sites(costs, w)
        assert shard.imbalance(costs, a) < 1.10
