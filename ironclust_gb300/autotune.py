"""Autotuner of the tensor-core kNN's work layout and tile shape.

The tensor-core kNN (irc_site_knn in IRC_MODE_BF16 / FP8) serves work items:
128 queries of a large chunk, or the remainders of up to max_slots small
chunks packed side by side (irc_plan_tc_layout), each item's candidates
streamed in units of 256 or 128 candidates (irc_plan_tc_units: the MMA width
N of the one- and two-slot items, with two or four accumulators in TMEM).
Which packing, item order and unit width are fastest depends on the feature
dimension and on the chunk sizes (a probe-scale batch has thousands of
~20-query chunks, a single drift site a few hundred 2,000-query chunks), so
they are measured, not guessed: every candidate is timed on the plan itself
with CUDA events and the fastest is applied.  Results depend on none of them.

Decisions are cached per (device, form, feature dimension, chunk-size and
candidate-count buckets) in a JSON file ($IRC_TUNE_CACHE, default
~/.cache/ironclust_gb300/tc_layout.json) so later plans of the same shape
skip the timing.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np
import torch

from . import irc
from ._lib import check, lib

# (max_slots, order, unit width): the candidates tried, the default first
CANDIDATES = [(4, 0, 256), (2, 0, 256), (1, 0, 256), (4, 1, 256), (4, 0, 128), (2, 0, 128), (1, 0, 128),
              (4, 1, 128)]


def cache_path():
    return os.environ.get("IRC_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "ironclust_gb300",
                                                            "tc_layout.json")


def signature(plan, n_features, mode):
    """Bucketed shape of a plan: feature dimension, median queries per chunk
    (log2 bucket) and median candidates per chunk (log2 bucket)."""
    d = plan.d
    nq = np.asarray(d["nq"], np.int64)
    roff = np.asarray(d["roff"], np.int64)
    rn = np.asarray(d["rn"], np.int64)
    cs = np.concatenate([[0], np.cumsum(rn)])
    cand = cs[roff[1:]] - cs[roff[:-1]]
    qb = int(math.log2(max(1.0, float(np.median(nq)))))
    cb = int(math.log2(max(1.0, float(np.median(cand)))))
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return "%s|%s|D%d|q%d|c%d" % (dev, mode, int(n_features), qb, cb)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass                                          # a read-only home: tune again next time


def apply(plan, layout):
    """layout: (max_slots, order[, unit width]) -- a width left out is 256."""
    check(lib().irc_plan_tc_layout(plan.h, int(layout[0]), int(layout[1])), "irc_plan_tc_layout")
    width = int(layout[2]) if len(layout) > 2 else 256
    check(lib().irc_plan_tc_units(plan.h, width), "irc_plan_tc_units")


def time_layout(plan, F, layout, knn=30, mode="bf16", reps=2):
    """Mean ms of irc_site_knn on this plan with the given layout."""
    apply(plan, layout)
    irc.site_knn(plan, F, knn, mode)                  # warm-up (operand buffers, caches)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        irc.site_knn(plan, F, knn, mode)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(plan, F, knn=30, mode="bf16", reps=2, use_cache=True, candidates=None):
    """Pick and apply the fastest layout for this plan.  Returns
    dict(layout=(max_slots, order, unit width), ms={layout: ms} (empty when
    cached), key, cached)."""
    key = signature(plan, F.shape[1], mode)
    table = _load() if use_cache else {}
    if key in table:
        layout = tuple(table[key]["layout"])
        layout = layout + (256,) * (3 - len(layout))          # entries written before the width was tuned
        apply(plan, layout)
        return dict(layout=layout, ms={}, key=key, cached=True)
    times = {}
    for lay in (candidates or CANDIDATES):
        times[tuple(lay)] = time_layout(plan, F, lay, knn, mode, reps)
    best = min(times, key=times.get)
    apply(plan, best)
    if use_cache:
        table = _load()
        table[key] = dict(layout=list(best), ms={",".join(map(str, k)): v for k, v in times.items()})
        _store(table)
    return dict(layout=best, ms=times, key=key, cached=False)
