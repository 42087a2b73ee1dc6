"""Autotuner for the batched solver: per (GPU, element type, size bucket), the
number of right-hand sides one work item solves (8, 16 or 32).

Each bucket is timed on a synthetic batch of its own sizes (seeded, on the
device) with every candidate, through the persistent kernel; the fastest is
cached as JSON at $NLA_TUNE_CACHE (default ~/.cache/nextla_gb300/tune.json)
under {gpu name: {dtype: {bucket: cols}}}.
"""

from __future__ import annotations

import json
import os

from . import _lib
from .batched import BatchPlan, make_batch

CANDIDATES = (8, 16, 32)
DTYPE_NAMES = {"torch.float16": "f16", "torch.float32": "f32", "torch.float64": "f64"}


def cache_path() -> str:
    return os.environ.get("NLA_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "nextla_gb300",
                                                         "tune.json"))


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(dtype, device=None):
    """Cached cols_per_item list for this GPU and dtype, or None."""
    import torch

    name = torch.cuda.get_device_name(device)
    entry = _load(cache_path()).get(name, {}).get(DTYPE_NAMES[str(dtype)])
    if not entry:
        return None
    try:
        return [int(entry[str(b)]) for b in range(_lib.NLA_BATCH_BUCKETS)]
    except KeyError:
        return None


def tune(dtype, device, systems_per_bucket=256, m=64, reps=3, save=True):
    """Time every candidate per size bucket; return the chosen list."""
    import numpy as np
    import torch

    chosen, timings = [], {}
    for b in range(_lib.NLA_BATCH_BUCKETS):
        lo, hi = 16 << b, min(32 << b, 1025)
        rng = np.random.default_rng(100 + b)
        n = rng.integers(lo, hi, systems_per_bucket)
        ms = np.full(systems_per_bucket, m)
        A, B0, systems = make_batch(n, ms, dtype, device, seed=100 + b)
        best, best_t = None, None
        for c in CANDIDATES:
            if dtype == torch.float64 and c == 32 and n.max() > 768:
                continue  # over the shared-memory budget for the largest systems
            plan = BatchPlan(dtype, "L", "N", systems, cols_per_item=[c] * _lib.NLA_BATCH_BUCKETS)
            B = B0.clone()
            plan.solve(1.0, A, B, mode="persistent")
            torch.cuda.synchronize(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                plan.solve(1.0, A, B, mode="persistent")
            e1.record()
            torch.cuda.synchronize(device)
            t = e0.elapsed_time(e1) / reps
            plan.close()
            timings.setdefault(b, {})[c] = t
            if best_t is None or t < best_t:
                best, best_t = c, t
        chosen.append(best)
        del A, B0
    if save:
        path = cache_path()
        data = _load(path)
        name = torch.cuda.get_device_name(device)
        data.setdefault(name, {})[DTYPE_NAMES[str(dtype)]] = {str(b): c for b, c in enumerate(chosen)}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return chosen, timings
