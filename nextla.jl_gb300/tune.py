"""Autotuner for the batched solver: per (GPU, element type, size bucket), the
leaf order of the recursion (16, 32 or 64 rows) and the widest block of
right-hand sides a group takes (32, 64 or 128; Float64 at most 64).

Each bucket is timed on a synthetic batch of its own sizes (seeded, on the
device; right-hand sides uniform in 1..128 as in the benchmark workload) with
every candidate pair, through the persistent kernel; the fastest pair is
cached as JSON at $NLA_TUNE_CACHE (default ~/.cache/nextla_gb300/tune.json)
under {gpu name: {dtype: {bucket: {"cutoff": c, "cols": w}}}}.
"""

from __future__ import annotations

import json
import os

from . import _lib
from .batched import BatchPlan, make_batch

CUTOFFS = (16, 32, 64)
COLS = (32, 64, 128)
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
    """Cached (cutoff list, cols list) for this GPU and dtype, or None."""
    import torch

    name = torch.cuda.get_device_name(device)
    entry = _load(cache_path()).get(name, {}).get(DTYPE_NAMES[str(dtype)])
    if not entry:
        return None
    try:
        return ([int(entry[str(b)]["cutoff"]) for b in range(_lib.NLA_BATCH_BUCKETS)],
                [int(entry[str(b)]["cols"]) for b in range(_lib.NLA_BATCH_BUCKETS)])
    except (KeyError, TypeError):
        return None


def candidates(dtype):
    import torch

    cols = tuple(c for c in COLS if not (dtype == torch.float64 and c > 64))
    return [(c, w) for c in CUTOFFS for w in cols]


def tune(dtype, device, systems_per_bucket=256, reps=3, save=True):
    """Time every candidate per size bucket; return ((cutoffs, cols), timings)."""
    import numpy as np
    import torch

    cut, cols, timings = [], [], {}
    for b in range(_lib.NLA_BATCH_BUCKETS):
        lo, hi = 16 << b, min(32 << b, 1025)
        rng = np.random.default_rng(100 + b)
        n = rng.integers(lo, hi, systems_per_bucket)
        m = rng.integers(1, 129, systems_per_bucket)
        A, B0, systems = make_batch(n, m, dtype, device, seed=100 + b)
        best, best_t = None, None
        for c, w in candidates(dtype):
            plan = BatchPlan(dtype, "L", "N", systems, cutoff=[c] * _lib.NLA_BATCH_BUCKETS,
                             cols=[w] * _lib.NLA_BATCH_BUCKETS)
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
            timings.setdefault(b, {})["%d/%d" % (c, w)] = t
            if best_t is None or t < best_t:
                best, best_t = (c, w), t
        cut.append(best[0])
        cols.append(best[1])
        del A, B0
    if save:
        path = cache_path()
        data = _load(path)
        name = torch.cuda.get_device_name(device)
        data.setdefault(name, {})[DTYPE_NAMES[str(dtype)]] = {
            str(b): {"cutoff": cut[b], "cols": cols[b]} for b in range(_lib.NLA_BATCH_BUCKETS)}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return (cut, cols), timings
