"""Launch-shape and threads-per-environment autotuner.

For a heterogeneous batch the tuner times, with CUDA events (median of a few launches
after warm-up):
  1. every launch shape: persistent CTAs per SM x warps per CTA x tile order (descending
     DoF / input order), one lane per environment;
  2. lanes per environment (1, 2, 4, 8) for each model in turn, largest tree first, each
     count with every launch shape, keeping the best pair (coordinate descent over the
     models): a team of L lanes shares one environment, the joints near the root on every
     lane and the subtrees off them split among the lanes, which shortens a wide tree's
     sequential sweep but needs more warps, hence the joint search with the shape;
  3. the five fastest (shape, lanes) pairs again with 20 launches each: the top candidates
     are often within a few percent, about the noise of a five-launch median.
The choice is cached in a JSON file keyed by GPU name, the batch signature (velocity
dimension, joint count and environment count of every model) and the op set, so a process
pays for the search once per tree mix.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

CANDIDATES = [(c, w, o) for o in (0, 1) for c in (1, 2, 4, 8) for w in (1, 2, 4) if c * w <= 16]


def _cache_path():
    d = os.environ.get("SGDYN_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "sapien_gb300")
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, "autotune.json")


def batch_signature(batch, ops):
    counts = np.bincount(batch.model_of_env, minlength=len(batch.models))
    parts = sorted((m.nv, m.njoints, int(c)) for m, c in zip(batch.models, counts))
    return f"ops{ops}:" + ",".join(f"nv{a}j{b}x{c}" for a, b, c in parts)


def _time(fn, reps=5):
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def tune_batch(batch, q, qd, qdd, tau, ops, use_cache=True, candidates=None, lane_candidates=(1, 2, 4, 8)):
    """Pick the fastest launch shape and lanes per environment for `batch` on these inputs,
    apply them to the batch and return (shape, table); the lanes are in batch.lanes."""
    key = f"{torch.cuda.get_device_name(batch.device)}|{batch_signature(batch, ops)}|lanes{tuple(lane_candidates)}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
    if use_cache and key in cache:
        shape = tuple(cache[key]["shape"])
        batch.set_launch(*shape)
        batch.set_lanes(cache[key].get("lanes", [1] * len(batch.models)))
        return shape, cache[key]["table"]
    out = batch.alloc_outputs(ops)
    shapes = list(candidates or CANDIDATES)
    table = []

    def measure(shape, lanes, reps=5, record=True):
        batch.set_launch(*shape)
        batch.set_lanes(lanes)
        ms = _time(lambda: batch.step(q, qd, qdd, tau, ops, out), reps=reps)
        if record:
            table.append({"shape": list(shape), "lanes": list(lanes), "ms": ms})
        return ms

    lanes = [1] * len(batch.models)
    best_ms, best_shape = min((measure(sh, lanes), sh) for sh in shapes)
    if len(lane_candidates) > 1:
        for m in sorted(range(len(batch.models)), key=lambda k: -batch.models[k].nv):
            for L in lane_candidates:
                if L == lanes[m]:
                    continue
                trial = lanes[:m] + [L] + lanes[m + 1:]
                ms, sh = min((measure(sh, trial), sh) for sh in shapes)
                if ms < best_ms:
                    best_ms, best_shape, lanes = ms, sh, trial
    top, seen = [], set()
    for r in sorted(table, key=lambda r: r["ms"]):
        k = (tuple(r["shape"]), tuple(r["lanes"]))
        if k not in seen:
            seen.add(k)
            top.append(k)
        if len(top) == 5:
            break
    if len(top) > 1:
        best_ms, best_shape, lanes = min((measure(sh, list(ln), reps=20, record=False), sh, list(ln))
                                         for sh, ln in top)
    batch.set_launch(*best_shape)
    batch.set_lanes(lanes)
    cache[key] = {"shape": list(best_shape), "lanes": lanes, "table": table, "when": time.time()}
    if use_cache:
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    return tuple(best_shape), table
