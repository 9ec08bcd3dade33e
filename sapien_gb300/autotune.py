"""Launch-shape autotuner.

For a heterogeneous batch the tuner times every candidate of
  persistent CTAs per SM  x  warps per CTA  x  tile order (descending DoF / input order)
with CUDA events (median of a few launches after warm-up) and keeps the fastest. Results
are cached in a JSON file keyed by GPU name, the batch signature (velocity dimension and
count of every model) and the op set, so a process pays for the search once per tree mix.
One environment runs per thread in every candidate (the per-lane work of the sweep is
sequential along the tree); the tile is one warp of environments of one model.
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


def tune_batch(batch, q, qd, qdd, tau, ops, use_cache=True, candidates=None):
    """Pick the fastest launch shape for `batch` on these inputs; returns (shape, table)."""
    key = f"{torch.cuda.get_device_name(batch.device)}|{batch_signature(batch, ops)}"
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
        return shape, cache[key]["table"]
    out = batch.alloc_outputs(ops)
    table = []
    for shape in candidates or CANDIDATES:
        batch.set_launch(*shape)
        ms = _time(lambda: batch.step(q, qd, qdd, tau, ops, out))
        table.append({"shape": list(shape), "ms": ms})
    best = min(table, key=lambda r: r["ms"])
    batch.set_launch(*best["shape"])
    cache[key] = {"shape": best["shape"], "table": table, "when": time.time()}
    if use_cache:
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    return tuple(best["shape"]), table
