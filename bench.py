"""Benchmark of the clustering hot path: kNN + rho + delta spikes/s.

One step = the whole hot path (kNN over the drift-linked candidates, rho =
1/d_knn, delta + nearest higher-rho spike) over one site of the
``drift400k`` workload: 400,000 spikes, 33 features, 16 Gaussian clusters,
200 drift chunks of ~2,000 spikes with a random-walk drift, each chunk
linked to its 15 most similar chunks within +/-64, knn = 30 (seeded
synthetic data: the recorded SpikeForest probes the reference measures on
are not available).

value : spikes/s of the headline form (inputs resident in HBM, L2 flushed
        before every timed step, CUDA events on the launching stream).
e2e   : the same through the public API with host buffers: H2D copy of the
        features from pinned memory + the site call + D2H copy of rho, delta,
        nneigh and the kNN list, every step.
forms : spikes/s of every form measured in the same run (the plain FP32
        drop-in "ref" form is the reference kernels' semantics bit for bit).

Multi-GPU: every rank runs an independent drift400k site (sites shard with
no exchange), value = all ranks' spikes / max-over-ranks time ("weak").  The
probe-scale batch splits its 384 sites over the ranks by LPT share
(shard.batch_share; strong scaling over the fixed probe) and rank 0 checks
the merged shares against one process running the whole probe.

--impl reference: the reference's CPU path (knn_cpu_ + delta_cpu_, irc2
with fGpu=0) restated in C with OpenMP, all host cores, on a bounded sample
of query chunks of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "kNN+rho+delta spikes/s: BF16-TC vs FP32 form on one GB300 at >=99.9% kNN recall"
WORKLOAD = "drift400k"
KNN = 30
MIN_COUNT = 30          # min_count of the reference's default parameters (matlab/default.prm:120)
TC_KNN_TRAFFIC_BYTES = 130.67e6 + 59.72e6    # ncu, one k_knn_tc launch on drift400k (read + write)
# ncu, the one-slot k_knn_tc launch of a middle block of the 100M-spike stream
STREAM_FILTER_NCU = {"kernel": "k_knn_tc<0, 256, 1, 1>", "duration_ms": 0.698,
                     "tensor_pipe_active_pct": 12.04, "dram_read_bytes": 124.71e6, "dram_write_bytes": 68.52e6,
                     "dram_throughput_pct": 3.49, "source": "profiles/launches_stream100m.md"}


def _dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return dict(hbm=p["hbm_gbs"], bf16=p["bf16_tflops"], bf16_sus=p["bf16_tflops_sustained"],
                    src="measured")
    except Exception:
        return dict(hbm=6800.0, bf16=1900.0, bf16_sus=1700.0, src="fallback")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(rank, scale):
    from ironclust_gb300 import synth
    site = synth.make_workload(WORKLOAD, scale=scale, seed_offset=rank)
    plan = synth.site_plan(site)
    return site, plan


def run_ours(args):
    import torch
    import torch.distributed as dist

    from ironclust_gb300 import _lib, build, irc
    from ironclust_gb300.drift import plan_pairs

    rank, world, local = _dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    build.build()
    _lib.lib()
    site, plan = make_inputs(rank, args.scale)
    N, D = site["F"].shape
    pairs = plan_pairs(plan)
    F = torch.from_numpy(site["F"]).to(dev)
    P = irc.Plan(plan)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)     # > L2 (126 MB)
    stream = torch.cuda.current_stream()

    forms = [m.strip() for m in args.forms.split(",") if m.strip()]
    head = args.mode if args.mode in forms else forms[0]
    results = {}
    kernel_ms = {}
    launch_ms = {}
    from ironclust_gb300 import autotune
    tuned = {}
    for mode in forms:
        if mode in ("bf16", "fp8"):
            t = autotune.tune(P, F, KNN, mode, use_cache=False)
            tuned[mode] = {"layout": {"max_slots": t["layout"][0], "order": t["layout"][1], "unit_width": t["layout"][2]},
                           "knn_ms": {",".join(map(str, k)): v for k, v in t["ms"].items()}}

        def step():
            return irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)
        try:
            for _ in range(args.warmup):
                step()
            torch.cuda.synchronize()
        except _lib.IrcError as e:
            results[mode] = {"error": str(e)}
            continue
        times = []
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        # the tensor-core forms time their filter and re-rank kernels with
        # CUDA events on the launch stream during the timed steps
        prof = mode in ("bf16", "fp8")
        if prof:
            _lib.check(_lib.lib().irc_profile_begin(args.steps + 1), "irc_profile_begin")
        with ClockSampler(dev.index) as cs:
            for _ in range(args.steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step()
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if prof:
            fa, fb, nc = ctypes.c_float(), ctypes.c_float(), ctypes.c_int()
            _lib.check(_lib.lib().irc_profile_end(ctypes.byref(fa), ctypes.byref(fb), ctypes.byref(nc)),
                       "irc_profile_end")
            launch_ms[mode] = {"k_knn_tc": fa.value / max(nc.value, 1), "k_rerank": fb.value / max(nc.value, 1),
                               "launches": nc.value}
        ms = sum(times) / len(times)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        results[mode] = {"spikes_per_s": world * N / (ms / 1e3), "ms_per_step": ms,
                         "clocks": cs.summary()}
        kernel_ms[mode] = time_kernels(P, F, mode, stream, flush, torch, irc)

    # accuracy of the headline form against the FP64 oracle is measured in the
    # tests; here the recall of each form is checked against the EXACT form
    # (whose kNN equals the FP32 oracle bit for bit) on the full workload.
    recall = {}
    if "exact" in forms and not results.get("exact", {}).get("error"):
        ref = irc.site_knn(P, F, KNN, "exact")["miKnn"]
        for mode in forms:
            if mode in ("exact",) or results.get(mode, {}).get("error"):
                continue
            got = irc.site_knn(P, F, KNN, mode)["miKnn"]
            recall[mode] = knn_recall(ref, got, torch)

    # accuracy of every form against the FP64 oracle on every spike of the
    # workload (outside the timed region; the oracle is the checker)
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        accuracy = accuracy_vs_fp64(P, F, site, plan, forms, results, torch, irc)

    # end-to-end through host buffers (headline form)
    e2e = None
    if not results.get(head, {}).get("error"):
        e2e = time_e2e(P, site["F"], head, args, dev, torch, irc, world, dist if world > 1 else None)
    post = None
    if rank == 0 and not results.get(head, {}).get("error"):
        post, post_inputs = run_post_cluster(P, F, head, args, torch, irc, stream, flush)
    streamed = None
    if args.stream100m and rank == 0:
        streamed = run_stream(args, dev, torch, irc)
    batched = None
    if args.batched:
        del F
        P.close()
        batched = run_batched(args, dev, torch, irc, flush, stream, dist if world > 1 else None)
        P = None

    out = None
    if rank == 0:
        peaks = _peaks()
        hr = results.get(head, {})
        km = kernel_ms.get(head, {})
        dom_name, dom_ms = (max(km.items(), key=lambda kv: kv[1]) if km else (None, None))
        flops = 2.0 * D * pairs
        roof = None
        if dom_ms:
            if head in ("bf16", "fp8") and launch_ms.get(head):
                # the dominant kernel is the filter, k_knn_tc: its average
                # launch time over the timed steps (CUDA events on its stream)
                tc_ms = launch_ms[head]["k_knn_tc"]
                mma_fpp = 2 * 2 * (32 * ((D + 12 + 31) // 32) if head == "fp8" else 16 * ((D + 9 + 15) // 16))
                ach = flops / (tc_ms / 1e3) / 1e12
                # DRAM bytes (read + write) of one launch of k_knn_tc on this
                # exact workload, captured once with ncu
                # (dram__bytes_read.sum + dram__bytes_write.sum).
                traffic = TC_KNN_TRAFFIC_BYTES if (args.scale == 1.0 and world == 1) else None
                roof = {"bound": "tensor", "kernel": "k_knn_tc", "achieved": ach,
                        "peak": peaks["bf16"], "unit": "TFLOP/s", "frac": ach / peaks["bf16"],
                        "traffic": traffic, "traffic_unit": "bytes per launch",
                        "launch_ms": tc_ms, "launches_timed": launch_ms[head]["launches"],
                        "hbm_gbs_at_traffic": (traffic / (tc_ms / 1e3) / 1e9) if traffic else None,
                        "hbm_peak_gbs": peaks["hbm"],
                        "flops_per_pair": 2 * D,
                        # the MMA work behind it: two passes over K values per pair (features, norm
                        # and threshold terms; BF16: 16 per slice, FP8: 32), tile padding excluded
                        "mma_flops_per_pair": mma_fpp,
                        "mma_tflops_issued": mma_fpp * pairs / (tc_ms / 1e3) / 1e12,
                        "peak_src": peaks["src"] + " bf16 burst"}
            else:
                ach = flops / (dom_ms / 1e3) / 1e12
                fp32_peak = 2 * 128 * 152 * 2.07e9 / 1e12        # FP32 SIMT FMA, nominal
                roof = {"bound": "fp32-simt", "kernel": dom_name, "achieved": ach, "peak": fp32_peak,
                        "unit": "TFLOP/s", "frac": ach / fp32_peak, "traffic": None,
                        "peak_src": "nominal 152 SM x 128 lanes x 2.07 GHz"}
        n_launch = {"ref": 2, "exact": 6, "bf16": 10, "fp8": 11}
        out = {
            "metric": METRIC, "value": hr.get("spikes_per_s"), "unit": "spikes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": hr.get("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"bf16": "bf16", "fp8": "fp8-e4m3", "exact": "f32", "ref": "f32"}.get(head, "f32"),
            "data": "synthetic (seeded Gaussian clusters + 5% noise, random-walk drift)",
            "config": {"workload": WORKLOAD, "spikes_per_site": N, "features": D, "chunks": len(plan["q0"]),
                       "links_per_chunk": 15, "knn": KNN, "form": head, "pairs": pairs,
                       "parallelism": "sites sharded over ranks" if world > 1 else "single site",
                       "l2": "flushed (256 MB write) before every timed step"},
            "forms": {m: {k: v for k, v in r.items() if k != "clocks"} for m, r in results.items()},
            "kernel_ms": kernel_ms,
            "launch_ms": launch_ms,
            "autotune": tuned,
            "recall_vs_exact": recall,
            "accuracy_vs_fp64": accuracy,
            "clocks": hr.get("clocks"),
            "e2e": e2e,
            "roofline": roof,
            "gpu_launches": n_launch.get(head, 0) * args.steps,
        }
        if "fp8" in out["forms"]:
            out["forms"]["fp8"]["note"] = ("not a headline form: e4m3 precision caps the filter's recall below 99.9% "
                                           "(0.98 with ~90-candidate lists; oracle/fp8_ceiling.py)")
        if accuracy and head in accuracy:
            out["recall_vs_fp64"] = accuracy[head]["recall_vs_fp64"]
            out["rho_max_rel_err"] = accuracy[head]["rho_max_rel_err"]
            out["delta_max_rel_err"] = accuracy[head]["delta_max_rel_err"]
        if batched is not None:
            out["batched"] = batched
        if streamed is not None:
            out["stream100m"] = streamed
        if post is not None:
            out["post_cluster"] = post
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(site, plan, seconds=args.cpu_seconds)
            if post is not None:
                post["cpu_baseline"] = post_cluster_cpu_baseline(post_inputs)
    if P is not None:
        P.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return out


def accuracy_vs_fp64(P, F, site, plan, forms, results, torch, irc):
    """kNN recall, rho and delta error of every form against the FP64 oracle
    on every spike (oracle.accuracy: delta from the FP64 rho; a different
    nearest higher-rho neighbour is an error unless FP32 and FP64 rho order
    the two candidates differently, counted apart as rho-order flips)."""
    from oracle import accuracy as A
    t0 = time.perf_counter()
    ref = A.fp64_reference(site["F"], plan, KNN)
    res = {"fp64_seconds": time.perf_counter() - t0}
    for mode in forms:
        if results.get(mode, {}).get("error"):
            continue
        o = irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)
        res[mode] = A.compare({k: v.cpu().numpy() for k, v in o.items() if v is not None}, ref)
    return res


def min_time_roofline(flops, nbytes, ms, peaks):
    """Roofline of a small-tile workload: the minimum time is the larger of
    its algorithmic flops at the sustained BF16 tensor rate and its
    compulsory bytes at the HBM rate; frac = that minimum / the measured
    time.  Both terms are reported."""
    t_tc = flops / (peaks["bf16_sus"] * 1e12) * 1e3
    t_hbm = nbytes / (peaks["hbm"] * 1e9) * 1e3
    return {"flops": flops, "bytes": nbytes, "t_tensor_ms": t_tc, "t_hbm_ms": t_hbm,
            "bound": "tensor" if t_tc >= t_hbm else "hbm", "min_ms": max(t_tc, t_hbm), "measured_ms": ms,
            "frac": max(t_tc, t_hbm) / ms, "peaks": "%s: bf16 sustained %.1f TFLOP/s, HBM %.1f GB/s" % (
                peaks["src"], peaks["bf16_sus"], peaks["hbm"])}


def run_batched(args, dev, torch, irc, flush, stream, dist=None):
    """The probe-scale batch (384 sites, 10M spikes, D in {18, 24, 33}, 1,200
    drift chunks): all sites in one plan, one launch per kernel, the whole
    kNN + rho + delta sequence captured in a CUDA graph and replayed.

    Under torchrun every rank builds the same probe, takes its LPT share of
    the sites (shard.batch_share) and runs that sub-batch; the step time is
    the maximum over ranks and the throughput all the probe's spikes / that
    time (strong scaling: the probe is fixed).  After the timed steps rank 0
    gathers the shares' outputs over a gloo group, merges them by global
    spike id (shard.gather_merge) and checks them against one process
    running the whole probe, bit for bit."""
    from ironclust_gb300 import shard, synth
    from ironclust_gb300.drift import plan_pairs
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist else (0, 1)
    t0 = time.perf_counter()
    b, specs = synth.make_probe(n_sites=args.probe_sites, total=args.probe_spikes)
    gen_s = time.perf_counter() - t0
    N = b.F.shape[0]
    if world > 1:
        mine, work = shard.batch_share(b, rank, world)
        cpu_group = dist.new_group(backend="gloo")
    else:
        mine, work = list(range(b.n_sites)), b
    F = torch.from_numpy(work.F).to(dev)
    P = work.make_plan()
    res = {"workload": "probe10m" if args.probe_sites == 384 else "probe%d" % args.probe_sites,
           "sites": b.n_sites, "spikes": N, "chunks": int(len(b.plan["q0"])), "pairs": plan_pairs(b.plan),
           "dims": sorted(set(int(d) for d in b.dims)), "generation_s": gen_s, "forms": {}}
    if world > 1:
        costs = shard.batch_costs(b)
        res["sharding"] = {"ranks": world, "scaling": "strong",
                           "sites_per_rank": [len(a) for a in shard.assign_sites(costs, world)],
                           "cost_imbalance": shard.imbalance(costs, shard.assign_sites(costs, world)),
                           "what": "LPT share of the sites per rank (shard.batch_share), no data-path "
                                   "collective; step time = max over ranks"}
    # algorithmic work: 2*D_site flops per pair (each site at its own D); compulsory bytes: every
    # site's features read once (4*D_site each) + the outputs (knn indices and d2, rho, delta, nneigh)
    pl = b.plan
    roff, rn = np.asarray(pl["roff"], np.int64), np.asarray(pl["rn"], np.int64)
    csum = np.concatenate([[0], np.cumsum(rn)])
    ncand = csum[roff[1:]] - csum[roff[:-1]]
    dsite = np.asarray(b.dims, np.int64)[np.asarray(b.site_of_chunk)]
    alg_flops = float(np.sum(2 * dsite * np.asarray(pl["nq"], np.int64) * ncand))
    alg_bytes = float(np.sum(np.asarray(b.sizes) * np.asarray(b.dims) * 4) + N * (KNN * 8 + 12))
    peaks = _peaks()
    from ironclust_gb300 import autotune
    outs, kept = {}, {}
    # whole sites drawn (seeded) until they hold >= 1 M spikes: the FP64 check's subsample
    picked, total = [], 0
    for s in np.random.default_rng(2024).permutation(b.n_sites):
        picked.append(int(s))
        total += int(b.sizes[s])
        if total >= 1_000_000:
            break

    def max_over_ranks(ms):
        if world == 1:
            return ms
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed(fn):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        times = []
        for _ in range(args.batched_steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        return max_over_ranks(sum(times) / len(times))

    for mode in [m.strip() for m in args.batched_forms.split(",") if m.strip()]:
        tuned = None
        if mode in ("bf16", "fp8"):
            t = autotune.tune(P, F, KNN, mode, use_cache=False)
            tuned = {"layout": {"max_slots": t["layout"][0], "order": t["layout"][1], "unit_width": t["layout"][2]},
                     "knn_ms": {",".join(map(str, k)): v for k, v in t["ms"].items()}}
        for _ in range(2):
            irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)
        torch.cuda.synchronize()
        ms_e = timed(lambda: irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode))
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)      # warm on the capture stream
        torch.cuda.current_stream().wait_stream(side)
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            out = irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)
        ms_g = timed(g.replay)
        res["forms"][mode] = {"ms_eager": ms_e, "ms_graph": ms_g, "spikes_per_s_graph": N / (ms_g / 1e3),
                              "spikes_per_s_eager": N / (ms_e / 1e3),
                              "roofline": min_time_roofline(alg_flops, alg_bytes, ms_g, peaks)}
        if tuned:
            res["forms"][mode]["autotune"] = tuned
        keys = ("miKnn", "rho", "delta", "nneigh")
        if world > 1:
            host = {k: out[k].cpu().numpy() for k in keys}
            merged = shard.gather_merge(b, mine, host, rank, world, cpu_group)
            if rank == 0:
                Pw, Fw = b.make_plan(), torch.from_numpy(b.F).to(dev)
                whole = irc.knn_rho_delta_site(Pw, Fw, knn=KNN, mode=mode)
                same = all(np.array_equal(merged[k].view(np.int32), whole[k].cpu().numpy().view(np.int32))
                           for k in keys)
                res["forms"][mode]["sharded_equals_one_process"] = bool(same)
                Pw.close()
                del Fw, whole
                outs[mode] = torch.from_numpy(merged["miKnn"])
                kept[mode] = {k: np.concatenate([merged[k][b.site_slice(s)] for s in picked]) for k in keys}
        else:
            outs[mode] = out["miKnn"].clone()
            kept[mode] = {k: torch.cat([out[k][b.site_slice(s)] for s in picked]).cpu().numpy() for k in keys}
        del g
    P.close()
    if rank != 0:
        return None
    if "exact" in outs:
        for mode, mi in outs.items():
            if mode != "exact":
                res["forms"][mode]["recall_vs_exact"] = knn_recall(outs["exact"], mi, torch)
    if not args.no_accuracy and kept:
        t0 = time.perf_counter()
        res["accuracy_sample"] = {"sites": len(picked), "spikes": total,
                                  "what": "whole sites drawn with a seeded permutation until >= 1 M spikes"}
        res["accuracy_vs_fp64"] = batch_accuracy(b, picked, kept, KNN)
        res["accuracy_sample"]["fp64_seconds"] = time.perf_counter() - t0
    return res


def batch_accuracy(b, picked, kept, knn):
    """Accuracy of each batched form on the picked sites against the FP64
    oracle (site by site, aggregated over all checked spikes)."""
    from oracle import accuracy as A
    refs = [A.fp64_reference(np.ascontiguousarray(b.F[b.site_slice(s), :int(b.dims[s])]), b.site_plans[s], knn)
            for s in picked]
    res = {}
    for mode, o in kept.items():
        stats, off = [], 0
        for s, ref in zip(picked, refs):
            n, base = int(b.sizes[s]), int(b.bases[s])
            part = {k: v[off:off + n] for k, v in o.items()}
            part["miKnn"] = part["miKnn"] - base
            part["nneigh"] = part["nneigh"] - base
            stats.append(A.compare(part, ref))
            off += n
        n = sum(x["checked"] for x in stats)
        res[mode] = {"checked": n,
                     "recall_vs_fp64": sum(x["recall_vs_fp64"] * x["checked"] for x in stats) / n,
                     "rho_max_rel_err": max(x["rho_max_rel_err"] for x in stats),
                     "delta_max_rel_err": max(x["delta_max_rel_err"] for x in stats),
                     "nneigh_errors": sum(x["nneigh_errors"] for x in stats),
                     "nneigh_rho_order_flips": sum(x["nneigh_rho_order_flips"] for x in stats)}
    return res


def run_stream(args, dev, torch, irc):
    """The multi-day shape streamed from pinned host memory (FP16 features,
    blocks of 128 drift chunks through a five-block device ring, copies
    overlapped with compute on three streams): end-to-end spikes/s from the
    first copy in to the last copy out, and recall, rho and delta error
    against the FP64 oracle on one whole block in the middle of the
    recording (1.27 M spikes)."""
    from ironclust_gb300 import stream
    t0 = time.perf_counter()
    wl = stream.make_workload(total=args.stream_spikes)
    gen_s = time.perf_counter() - t0
    st = stream.Streamer(wl, knn=KNN, mode="bf16")
    st.run()                                           # warm-up: plan buffers, caches
    ms = [st.run() for _ in range(2)]
    N = int(wl["block_base"][-1])
    h2d, d2h = st.bytes_per_pass()
    res = {"workload": "stream%dm" % round(N / 1e6), "spikes": N, "sites": len(wl["sizes"]),
           "chunks": wl["n_chunks"], "features": wl["n_dim"], "blocks": wl["n_blocks"],
           "pairs": int(sum(plan_pairs_of(p) for p in st.plans)), "generation_s": gen_s,
           "ms": sum(ms) / len(ms), "spikes_per_s": N / (sum(ms) / len(ms) / 1e3),
           "h2d_bytes": h2d, "d2h_bytes": d2h,
           "host_link_gbs": (h2d + d2h) / (sum(ms) / len(ms) / 1e3) / 1e9,
           "data": "synthetic: FP16 features in pinned host memory, random-walk + 0.01/step drift"}
    # roofline of the device work: 2*D flops per pair; compulsory device bytes: the FP16 features in,
    # widened once, and the outputs
    D = wl["n_dim"]
    res["roofline"] = min_time_roofline(2.0 * D * res["pairs"], float(N * D * (2 + 4) + N * (KNN * 4 + 12)),
                                        res["ms"], _peaks())
    r = res["roofline"]
    # device throughput of the pass: the compulsory device bytes (FP16 features in, widened once,
    # outputs) and the issued BF16 MMA work per second; the DRAM bytes and tensor-pipe activity ncu
    # measured on a streamed block are in the committed stream profile
    res["hbm_gbs_compulsory"] = r["bytes"] / (res["ms"] / 1e3) / 1e9
    res["tensor_tflops_algorithmic"] = r["flops"] / (res["ms"] / 1e3) / 1e12
    res["tensor_frac_algorithmic"] = res["tensor_tflops_algorithmic"] / _peaks()["bf16"]
    # counters of one middle block's one-slot filter launch, from a separate ncu capture of the same
    # streamed pass (never a number taken under the profiler in this run)
    res["ncu_filter_launch"] = STREAM_FILTER_NCU
    if not args.no_accuracy:
        # accuracy against FP64 on the middle block (>= 1 M spikes of the recording): kNN recall,
        # rho and delta with nearest higher-rho neighbours (oracle.accuracy.stream_block_check)
        from oracle import accuracy as A
        t0 = time.perf_counter()
        acc = A.stream_block_check(st, wl["n_blocks"] // 2, KNN)
        acc["fp64_seconds"] = time.perf_counter() - t0
        res["accuracy_vs_fp64"] = acc
        res.update(recall_vs_fp64=acc["recall_vs_fp64"], rho_max_rel_err=acc["rho_max_rel_err"],
                   delta_max_rel_err=acc["delta_max_rel_err"], nneigh_errors=acc["nneigh_errors"])
    st.close()
    return res


def plan_pairs_of(P):
    from ironclust_gb300.drift import plan_pairs
    return plan_pairs(P.d)


def knn_recall(ref, got, torch):
    r = ref.long()
    g = got.long()
    n = r.shape[0]
    hits = 0
    for s in range(0, n, 65536):
        a = r[s:s + 65536]
        b = g[s:s + 65536]
        hits += (a.unsqueeze(2) == b.unsqueeze(1)).any(2).sum().item()
    return hits / float(r.numel())


def time_kernels(P, F, mode, stream, flush, torch, irc):
    """Per-phase device times of one step (CUDA events on the launch stream)."""
    flush.zero_()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    k = irc.site_knn(P, F, KNN, mode)
    ev[1].record(stream)
    irc.site_delta(P, F, k["rho"], mode, 512, KNN, k["miKnn"], k["d2Knn"])
    ev[2].record(stream)
    ev[2].synchronize()
    return {"knn": ev[0].elapsed_time(ev[1]), "delta": ev[1].elapsed_time(ev[2])}


def time_e2e(P, F_host, mode, args, dev, torch, irc, world, dist):
    """The headline form through the public fused call with host buffers:
    every step copies its features from pinned host memory to the device,
    runs kNN -> rho -> delta (irc_knn_rho_delta_site) and copies rho, delta,
    nneigh and the kNN list back to pinned host memory, all inside the timed
    region.  Steps are pipelined as a host streaming many sites would run
    them: step k+1's features go up on a copy stream (two device buffers)
    while step k computes, and step k's results come down on a third stream."""
    Fh = torch.from_numpy(F_host).pin_memory()
    N = Fh.shape[0]
    Fd = [torch.empty_like(Fh, device=dev) for _ in range(2)]
    outs = {"rho": torch.empty(N, dtype=torch.float32).pin_memory(),
            "delta": torch.empty(N, dtype=torch.float32).pin_memory(),
            "nneigh": torch.empty(N, dtype=torch.int32).pin_memory(),
            "miKnn": torch.empty((N, KNN), dtype=torch.int32).pin_memory()}
    s_c = torch.cuda.current_stream()
    s_h, s_d = torch.cuda.Stream(), torch.cuda.Stream()

    def run(n):
        ev_in = [torch.cuda.Event() for _ in range(n)]
        ev_used = [torch.cuda.Event() for _ in range(n)]

        def upload(k):
            with torch.cuda.stream(s_h):
                if k >= 2:
                    s_h.wait_event(ev_used[k - 2])        # the buffer's previous step has computed
                Fd[k % 2].copy_(Fh, non_blocking=True)
                ev_in[k].record(s_h)

        upload(0)
        for k in range(n):
            if k + 1 < n:
                upload(k + 1)
            s_c.wait_event(ev_in[k])
            r = irc.knn_rho_delta_site(P, Fd[k % 2], knn=KNN, mode=mode)
            ev_used[k].record(s_c)
            with torch.cuda.stream(s_d):
                s_d.wait_event(ev_used[k])
                for key, h in outs.items():
                    r[key].record_stream(s_d)
                    h.copy_(r[key], non_blocking=True)
        s_c.wait_stream(s_d)

    s_h.wait_stream(s_c)
    run(max(1, args.warmup))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s_c)
    s_h.wait_event(e0)
    run(args.steps)
    e1.record(s_c)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    h2d = Fh.numel() * 4
    d2h = sum(h.numel() * h.element_size() for h in outs.values())
    return {"value": world * N / (ms / 1e3), "unit": "spikes/s", "ms_per_step": ms,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "pipelining": "step k+1's upload and step k's download overlap step k's compute (three streams)"}


def run_post_cluster(P, F, mode, args, torch, irc, stream, flush):
    """The clustering step after the path on the headline form's outputs:
    sort_'s normalisation (irc_sort_rho) and postCluster_'s assignment
    (irc_assign_cluster_knn), device time per step (CUDA events, L2 flushed
    before each step).  The step synchronises the host a few times (peak
    count, merge repeats, propagation passes), which the events include."""
    k = irc.knn_rho_delta_site(P, F, knn=KNN, mode=mode)
    N = F.shape[0]
    rho = k["rho"]
    # delta_paged_site_'s NaN/Inf rule and global ids (one page: identity)
    delta = k["delta"].clone()
    bad = ~torch.isfinite(delta)
    delta[bad] = float(irc.SQRT_SINGLE_INF_F)
    nneigh = torch.where(bad, torch.arange(1, N + 1, device=F.device), k["nneigh"].long())
    mk = k["miKnn"].long()

    def step():
        rn, order = irc.sort_rho(rho)
        return irc.assign_cluster_knn(rn, delta, order, nneigh, mk, 1.0, MIN_COUNT)

    for _ in range(max(1, args.warmup)):
        a = step()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        a = step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = sum(times) / len(times)
    host = dict(rho=rho.cpu().numpy(), delta=delta.cpu().numpy(), nneigh=nneigh.cpu().numpy(),
                miKnn=mk.cpu().numpy())
    return ({"workload": "%s, %s-form rho/delta/nneigh/kNN" % (WORKLOAD, mode), "steps": args.steps,
             "ms_per_step": ms, "spikes_per_s": N / (ms / 1e3), "delta_cut": 1.0, "min_count": MIN_COUNT,
             "peaks": a["nClu_pre"], "clusters_after_merge": a["nClu_post"], "clusters": a["nClu"]}, host)


def post_cluster_cpu_baseline(host):
    """The clustering step's CPU restatement (serial, as MATLAB's loops are)
    on the same inputs: one pass over the whole workload."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    r, o = O.sort_rho(host["rho"])
    O.assign_cluster_knn(r, host["delta"], o, host["nneigh"], host["miKnn"], 1.0, MIN_COUNT)
    t = time.perf_counter() - t0
    n = host["rho"].size
    return {"value": n / t, "unit": "spikes/s", "cores": 1, "kind": "port",
            "sample": "the whole workload, one pass (sort_ normalisation + postCluster_ assignment)",
            "seconds": t}


def cpu_baseline(site, plan, seconds=15.0, chunks=None):
    """The reference CPU path (knn_cpu_ + delta_cpu_, OpenMP, all host cores)
    over a bounded sample of query chunks; spikes/s of the sample."""
    from oracle import oracle as O
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    F = site["F"]
    rng = np.random.default_rng(0)
    R_stand_in = rng.uniform(0.05, 1.0, F.shape[0]).astype(np.float32)
    n_done, t_used, n_ch = 0, 0.0, 0
    n_total = len(plan["q0"])
    step = 1 if chunks is None else chunks
    while n_ch < n_total:
        take = min(step, n_total - n_ch)
        # the next `take` query chunks, with their own candidate runs
        new = dict(q0=plan["q0"][n_ch:n_ch + take], nq=plan["nq"][n_ch:n_ch + take],
                   roff=(plan["roff"][n_ch:n_ch + take + 1] - plan["roff"][n_ch]),
                   rs=plan["rs"][plan["roff"][n_ch]:plan["roff"][n_ch + take]],
                   rn=plan["rn"][plan["roff"][n_ch]:plan["roff"][n_ch + take]],
                   q_base=int(plan["q0"][n_ch]), n_out=int(plan["nq"][n_ch:n_ch + take].sum()),
                   n_f=plan["n_f"])
        t0 = time.perf_counter()
        vr, _ = O.site_knn_cpu(F, new, KNN)
        R = R_stand_in.copy()
        R[new["q_base"]:new["q_base"] + new["n_out"]] = 1.0 / vr
        O.site_delta_cpu(F, R, new)
        t_used += time.perf_counter() - t0
        n_done += new["n_out"]
        n_ch += take
        if chunks is None and t_used >= seconds:
            break
        if chunks is not None:
            break
    return {"value": n_done / t_used, "unit": "spikes/s", "cores": cores, "kind": "port",
            "sample": "%d query chunks (%d of %d spikes) of %s through knn_cpu_ + delta_cpu_ (C port, "
                      "OpenMP); rho of non-sampled candidates is a seeded stand-in" % (
                          n_ch, n_done, site["F"].shape[0], WORKLOAD),
            "seconds": t_used}


def reference_gpu_kernels(site, plan, passes=2):
    """The reference's own GPU kernels on this GB300, a same-box reference GPU
    number: search_min_drift and search_delta_drift (PTX compiled from the
    reference sources by oracle/build_oracle.py, launched through
    oracle/ref_harness.cu with MATLAB's launch configuration) once per query
    chunk, as search_knn_drift_ / search_delta_drift_ issue them
    (matlab/irc2.m:3752-3789, :3814-3860), with MATLAB's gpuArray sort / min
    stood in for by a stable device sort / min (torch).  Kernel and sort time
    only: MATLAB's interpreter and gpuArray bookkeeping are not counted."""
    import torch
    if not torch.cuda.is_available():
        return None
    from oracle import oracle as O
    try:
        refk = O.RefKernels()
    except Exception as e:                                   # PTX or harness missing on this machine
        return {"unavailable": str(e).splitlines()[0][:200]}
    F = torch.from_numpy(site["F"]).cuda()
    nF, nC = F.shape[0], F.shape[1]
    chunks = []
    for i in range(len(plan["q0"])):
        r0, r1 = int(plan["roff"][i]), int(plan["roff"][i + 1])
        chunks.append((torch.from_numpy(np.ascontiguousarray(plan["rs"][r0:r1])).cuda(),
                       torch.from_numpy(np.ascontiguousarray(plan["rn"][r0:r1])).cuda(),
                       [nC, nF, r1 - r0, int(plan["q0"][i]), int(plan["nq"][i])]))
    rho = torch.empty(nF, dtype=torch.float32, device="cuda")

    def one_pass():
        for IBB, NBB, vn in chunks:
            D, I = refk.search_min_drift(F, IBB, NBB, vn)
            vs, _ = torch.sort(D, dim=1, stable=True)
            rho[vn[3]:vn[3] + vn[4]] = 1.0 / vs[:, KNN - 1]
        for IBB, NBB, vn in chunks:
            D, I = refk.search_delta_drift(F, rho, IBB, NBB, vn)
            torch.min(D, dim=1)

    one_pass()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(passes):
        one_pass()
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / passes
    return {"ms_per_pass": ms, "spikes_per_s": nF / (ms / 1e3), "launches_per_pass": 2 * len(chunks),
            "what": "reference search_min_drift + search_delta_drift PTX, one launch per chunk, MATLAB launch "
                    "configuration; stable device sort / min standing in for MATLAB's gpuArray sort / min"}


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return None
    site, plan = make_inputs(0, args.scale)
    N = site["F"].shape[0]
    from oracle import oracle as O  # noqa: F401  (builds the oracle library)
    sample_chunks = args.ref_chunks
    for _ in range(args.warmup):
        cpu_baseline(site, plan, chunks=sample_chunks)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(site, plan, chunks=sample_chunks))
    wall = time.perf_counter() - t0
    v = sum(x["value"] for x in vals) / len(vals)
    ref_gpu = reference_gpu_kernels(site, plan)
    return {"reference_gpu_kernels": ref_gpu, "metric": METRIC, "value": v, "unit": "spikes/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic (seeded Gaussian clusters + 5% noise, random-walk drift)",
            "config": {"workload": WORKLOAD, "spikes_per_site": N, "knn": KNN,
                       "form": "reference CPU path (irc2 fGpu=0): knn_cpu_ + delta_cpu_"},
            "cpu_baseline": {k: vals[0][k] for k in ("kind", "cores", "sample")} | {"value": v, "unit": "spikes/s"},
            "e2e": {"value": v, "unit": "spikes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="bf16")
    ap.add_argument("--forms", default="bf16,fp8,exact,ref")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-chunks", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the accuracy checks against the FP64 oracle (run outside the timed regions)")
    ap.add_argument("--batched", dest="batched", action="store_true", default=True,
                    help="also time the probe-scale batch (all sites in one plan, CUDA graph)")
    ap.add_argument("--no-batched", dest="batched", action="store_false")
    ap.add_argument("--batched-forms", default="bf16,fp8,exact,ref")
    ap.add_argument("--batched-steps", type=int, default=3)
    ap.add_argument("--probe-sites", type=int, default=384)
    ap.add_argument("--probe-spikes", type=int, default=10_000_000)
    ap.add_argument("--stream100m", dest="stream100m", action="store_true", default=True,
                    help="also run the multi-day streaming shape (100M spikes, 384 sites, FP16 in pinned host "
                         "memory, 10,000 chunks); on by default")
    ap.add_argument("--no-stream100m", dest="stream100m", action="store_false")
    ap.add_argument("--stream-spikes", type=int, default=100_000_000)
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
