#!/usr/bin/env python
"""Benchmark of the recursive triangular solve on one GB300.

Workload (default): Float64 TRSM, side L, uplo L, trans N, alpha 1,
n = m = 16384, A = tril(N(0,1)/sqrt(n), -1) + diag(2 + |N(0,1)|),
B ~ U[-1, 1], seed 0 (numpy PCG64).  The inputs (2 GiB each) are larger than
L2 (129 MB), so no flush is needed between steps.

One step = restore B from a resident pristine copy (device-to-device copy,
inside the timed region) + one full solve.  Metric: TFLOP/s with the
n^2 m flop count of a triangular solve.

Variants:
  plain   the dtype-preserving Float64 path (DFMA GEMM updates, FP64 leaves).
  mixed   the mixed-precision form (default): every GEMM update on the BF16
          tensor cores.  With --terms 7 (default) each FP64 operand is split
          into 7 BF16 slices and the 28 significant slice pairs accumulate
          exactly (FP32 chunks drained into int64), so the updates are as
          accurate as FP64 and no refinement sweep is needed (--sweeps 0).
          --terms 1-3 with --sweeps >= 1 is the cheaper split plus
          FP64-residual iterative refinement.

Also reported on the same JSON line:
  e2e           the same metric through the C ABI with host buffers
                (nla_trxm_mixed_host / nla_trxm_host): pinned host A and B
                copied in, solved and X copied out every step, the copies
                pipelined with the recursion's top levels;
  roofline      the dominant kernel's achieved rate from live CUDA-event
                tracing inside the timed region against the measured peak;
  cpu_baseline  the oracle (a C restatement of the reference algorithm) on the
                host cores on a bounded sample of right-hand sides;
  clocks        nvidia-smi samples taken during the timed region.

--impl reference times the reference algorithm (the oracle port) on the host
cores on a bounded sample of the same workload, and prints the same metric.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", choices=["plain", "mixed"], default="mixed")
    ap.add_argument("--lowp", choices=["bf16", "f16"], default="bf16")
    ap.add_argument("--terms", type=int, default=7, help="split terms (1-3, or 7 for exact updates)")
    ap.add_argument("--sweeps", type=int, default=0)
    ap.add_argument("--residual", choices=["split", "fp64"], default="split")
    ap.add_argument("--cutoff", type=int, default=0)
    ap.add_argument("--host-levels", type=int, default=0,
                    help="recursion levels the host-buffer call pipelines its copies over (0: library default)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison step")
    ap.add_argument("--no-mixed", action="store_true", help="batched workload: skip the mixed-precision forms")
    ap.add_argument("--workload", choices=["single", "batched"], default="single",
                    help="single: one n x m system; batched: 10,000 uneven systems in one persistent launch")
    ap.add_argument("--dtype", choices=["f64", "f32"], default="f64", help="element type of the batched workload")
    ap.add_argument("--count", type=int, default=10000, help="systems in the batched workload")
    ap.add_argument("--tune", action="store_true", help="autotune the batched tile widths before timing")
    ap.add_argument("--error-table", action="store_true",
                    help="mixed-precision error and speed versus cond(A) (JSON line per configuration)")
    ap.add_argument("--conds", default="1e2,1e4,1e6,1e8")
    ap.add_argument("--error-variants", choices=["all", "exact"], default="all",
                    help="error table: every mixed configuration, or the default exact one only")
    ap.add_argument("--cpu-table", action="store_true",
                    help="time the CPU baselines of every configuration on this host: the oracle port of the "
                         "reference algorithm and OpenBLAS trsm/trmm through scipy, on all host threads")
    ap.add_argument("--config3", action="store_true",
                    help="mixed TRMM R/U/T n=12288 (3-term BF16) and Float16 TRSM n=8192 m=4096, vs FP64")
    ap.add_argument("--callers", action="store_true",
                    help="the package's own callers (LU's trsm, LAUUM's trmm updates) on the GPU path")
    ap.add_argument("--sweep-plain", action="store_true",
                    help="plain F32/F64 TRSM and TRMM over the 8 side/uplo/trans forms, alpha 0.5 (config 1)")
    ap.add_argument("--sizes", default="4096,8192,16384")
    ap.add_argument("--kernel-case", choices=["exact", "fast", "leaf", "pair", "dfma"], default=None,
                    help="run single launches of one kernel on a moderate case (for ncu captures)")
    ap.add_argument("--case-size", type=int, default=4096)
    ap.add_argument("--case-reps", type=int, default=2)
    ap.add_argument("--case-shape", default="",
                    help="M,N,K of the exact/fast update case (default: s,s,s); n,m of the leaf case")
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--m", type=int, default=16384)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="right-hand sides in the CPU sample (0: 128 per host thread)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (the GPU is not modified)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


PLAIN_STEPS = 3  # timed solves of the plain FP64 comparison
E2E_STEPS = 15   # synchronised end-to-end steps (host buffers to host result)

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# exact tensor-core kernel, averaged over the 127 updates of one default
# solve at n = m = 16384 (the 128 updates between sibling leaves run inside
# the leaf pair kernel).  ncu cannot run inside the timed bench, so this is
# the figure of one ncu capture of the same workload, with the commit and
# command it was taken on (TRAFFIC_SOURCE).
TRAFFIC_BYTES_PER_LAUNCH = 421.6e6
TRAFFIC_SOURCE = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none -k regex:umma_exact "
                  "-s 127 -c 127 python bench.py --steps 1 --warmup 1 --no-plain --no-cpu-baseline (the timed "
                  "solve's 127 updates), at commit 125abf4")


def make_inputs(n, m, seed=0):
    import numpy as np

    rng = np.random.default_rng(seed)
    A = np.tril(rng.standard_normal((n, n)) / np.sqrt(n), -1)
    A[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
    B = rng.uniform(-1.0, 1.0, (n, m))
    return np.asfortranarray(A), np.asfortranarray(B)


def cpu_baseline(A, B, sample_cols, threads):
    """Oracle (reference algorithm restated in C) on `sample_cols` right-hand
    sides with `threads` host threads; returns (TFLOP/s, seconds, columns)."""
    import numpy as np

    import __graft_entry__ as graft

    orc = graft.load_oracle()
    n = A.shape[0]
    Bs = np.asfortranarray(B[:, :sample_cols])
    t0 = time.perf_counter()
    orc.rectrxm("L", "L", "N", 1.0, "S", A, Bs, nthreads=threads)
    dt = time.perf_counter() - t0
    return float(n) * n * sample_cols / dt / 1e12, dt


def rank_env():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(ms, world, device):
    """The slowest rank's time.  Every rank times its own replica between the
    same barriers, and the job is done when the last one is."""
    if world <= 1:
        return ms
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_tflops(world, flops_per_rank, ms):
    """Whole-job rate: every rank does flops_per_rank in the slowest rank's ms."""
    return world * flops_per_rank / (ms / 1e3) / 1e12


def run_reference(args):
    """--impl reference: the reference algorithm (oracle port) on host cores.
    Under torchrun, rank 0 alone runs and prints; the other ranks exit."""
    _, rank, _ = rank_env()
    if rank != 0:
        return 0
    import numpy as np

    threads = os.cpu_count() or 1
    cols = args.cpu_sample or 128 * threads
    A, B = make_inputs(args.n, args.m)
    vals = []
    for i in range(args.warmup + args.steps):
        v, _ = cpu_baseline(A, B, cols, threads)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": "trsm_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
        "config": {"workload": "trsm_LLN_f64_n%d_m%d" % (args.n, args.m), "n": args.n, "m": args.m,
                   "side": "L", "uplo": "L", "trans": "N", "alpha": 1.0},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                         "sample": "%d of %d right-hand sides per step, full %dx%d A" % (cols, args.m, args.n,
                                                                                         args.n)},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_cpu_table(args):
    """CPU baselines of every configuration on this host's cores, one JSON
    line each: the oracle port of the reference algorithm (all threads) and
    OpenBLAS through scipy (its own thread pool, all cores).  Large cases time
    a bounded sample of right-hand sides (stated in the line); the rate is the
    sample's n^2 m flops over its time."""
    import numpy as np
    from scipy.linalg import blas

    import __graft_entry__ as graft

    orc = graft.load_oracle()
    threads = os.cpu_count() or 1

    def timed(fn, reps=2):
        fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps

    def tri(n, uplo, seed, dt=np.float64):
        rng = np.random.default_rng(seed)
        Z = rng.standard_normal((n, n)) / np.sqrt(n)
        A = np.tril(Z, -1) if uplo == "L" else np.triu(Z, 1)
        A[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
        return np.asfortranarray(A.astype(dt)), rng

    def line(cfg, impl, n, cols, secs, dtype, sample, func="S"):
        rec = {"config": cfg, "impl": impl, "dtype": dtype, "func": func, "n": n, "rhs": cols,
               "seconds": round(secs, 4), "gflops": round(float(n) * n * cols / secs / 1e9, 2),
               "threads": threads, "sample": sample}
        print(json.dumps(rec), flush=True)

    # 0: F64 TRSM L/L/N, n = 1024, m = 256
    A, rng = tri(1024, "L", 0)
    B = np.asfortranarray(rng.uniform(-1, 1, (1024, 256)))
    line(0, "oracle", 1024, 256, timed(lambda: orc.rectrxm("L", "L", "N", 1.0, "S", A, B, nthreads=threads)),
         "f64", "all")
    line(0, "openblas", 1024, 256, timed(lambda: blas.dtrsm(1.0, A, B, lower=1)), "f64", "all")
    # 1: plain TRSM/TRMM, B n x n (L/L/N shown; the other forms cost the same)
    for n in (4096, 8192, 16384):
        for dt, pre in ((np.float64, "d"), (np.float32, "s")):
            A, rng = tri(n, "L", 1, dt)
            cols = n if n <= 4096 else 2048
            Bs = np.asfortranarray(rng.uniform(-1, 1, (n, cols)).astype(dt))
            for func, fn in (("S", getattr(blas, pre + "trsm")), ("M", getattr(blas, pre + "trmm"))):
                line(1, "openblas", n, cols, timed(lambda: fn(0.5, A, Bs, lower=1), 1),
                     "f64" if pre == "d" else "f32", "all" if cols == n else "%d of %d columns" % (cols, n), func)
            if n == 4096:
                ocol = 256
                Bo = np.asfortranarray(Bs[:, :ocol])
                line(1, "oracle", n, ocol, timed(lambda: orc.rectrxm("L", "L", "N", 0.5, "S", A, Bo,
                                                                     nthreads=threads), 1),
                     "f64" if pre == "d" else "f32", "%d of %d columns" % (ocol, n))
    # 2: F64 TRSM n = m = 16384 (cond 1e2 .. 1e8 do not change the cost)
    A, rng = tri(16384, "L", 0)
    Bs = np.asfortranarray(rng.uniform(-1, 1, (16384, 2048)))
    line(2, "openblas", 16384, 2048, timed(lambda: blas.dtrsm(1.0, A, Bs, lower=1), 1), "f64",
         "2048 of 16384 columns")
    Bo = np.asfortranarray(Bs[:, :512])
    line(2, "oracle", 16384, 512, timed(lambda: orc.rectrxm("L", "L", "N", 1.0, "S", A, Bo, nthreads=threads), 1),
         "f64", "512 of 16384 columns")
    del A, Bs, Bo
    # 3: F64 TRMM R/U/T n = 12288; F16 TRSM n = 8192, m = 4096 (OpenBLAS in F32)
    A, rng = tri(12288, "U", 3)
    Bs = np.asfortranarray(rng.uniform(-1, 1, (2048, 12288)))
    line(3, "openblas", 12288, 2048, timed(lambda: blas.dtrmm(1.0, A, Bs, side=1, lower=0, trans_a=1), 1), "f64",
         "2048 of 12288 rows", "M")
    A, rng = tri(8192, "L", 4, np.float32)
    Bs = np.asfortranarray(rng.uniform(-1, 1, (8192, 4096)).astype(np.float32))
    line(3, "openblas", 8192, 4096, timed(lambda: blas.strsm(1.0, A, Bs, lower=1), 1), "f16 computed as f32", "all")
    del A, Bs
    # 4: 10,000 uneven systems, seed 7, one OpenBLAS call per system
    rng = np.random.default_rng(7)
    ns = np.clip(np.rint(np.exp(rng.uniform(np.log(16), np.log(1024), 10000))).astype(np.int64), 16, 1024)
    ms = rng.integers(1, 129, 10000)
    flops = float((ns.astype(float) ** 2 * ms).sum())
    for dt, pre in ((np.float64, "d"), (np.float32, "s")):
        systems = []
        for i in range(10000):
            Ai, r2 = tri(int(ns[i]), "L", 1000 + i % 64, dt)
            systems.append((Ai, np.asfortranarray(r2.uniform(-1, 1, (int(ns[i]), int(ms[i]))).astype(dt))))
        fn = getattr(blas, pre + "trsm")
        secs = timed(lambda: [fn(1.0, Ai, Bi, lower=1) for Ai, Bi in systems], 1)
        print(json.dumps({"config": 4, "impl": "openblas (one call per system)", "dtype": "f64" if pre == "d" else "f32",
                          "systems": 10000, "seconds": round(secs, 4), "gflops": round(flops / secs / 1e9, 2),
                          "threads": threads, "sample": "all"}), flush=True)
    return 0


def run_batched(args):
    """10,000 independent lower-triangular systems (side L, trans N), n_i
    log-uniform in [16, 1024], m_i uniform in 1..128, seed 7: one persistent
    launch replayed from a CUDA graph, against one recursion per system."""
    import torch

    import __graft_entry__ as graft

    graft.load_package()
    from nextla_gb300 import _lib, batched, tune

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    dtype = torch.float64 if args.dtype == "f64" else torch.float32
    n, m = batched.uneven_sizes(count=args.count, seed=7)
    A, B0, systems = batched.make_batch(n, m, dtype, dev, seed=7)
    flops = float((n.astype(float) ** 2 * m).sum())
    tuned = tune.tune(dtype, dev)[0] if args.tune else tune.lookup(dtype, dev)
    cutoff, cw = tuned if tuned else (None, None)
    plan = batched.BatchPlan(dtype, "L", "N", systems, cutoff=cutoff, cols=cw)
    B = B0.clone()
    stream = torch.cuda.current_stream(dev)

    def timed(mode, steps):
        for _ in range(args.warmup):
            B.copy_(B0)
            plan.solve(1.0, A, B, mode=mode)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            B.copy_(B0)
            plan.solve(1.0, A, B, mode=mode)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / steps

    _lib.trace_enable(True)
    ms = timed("graph", args.steps)
    _lib.trace_enable(False)
    trace = _lib.trace_summary()
    loop_ms = timed("loop", max(1, min(args.steps, 2)))
    items, grid, _ = plan.info()
    mixed = None
    if dtype == torch.float64 and not args.no_mixed:
        # Mixed-precision form: Float32 solves refined with Float64 residuals,
        # against the plain Float64 answer of the same batch.
        B.copy_(B0)
        plan.solve(1.0, A, B, mode="graph")
        X64 = B.clone()
        ref = float(torch.linalg.norm(X64))
        mixed = []
        for sweeps, res in ((0, "split"), (1, "split"), (2, "split"), (3, "split"), (2, "fp64")):
            def mstep():
                B.copy_(B0)
                plan.solve_mixed(1.0, A, B, sweeps=sweeps, residual=res)
            for _ in range(args.warmup):
                mstep()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                mstep()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            mms = e0.elapsed_time(e1) / args.steps
            mixed.append({"sweeps": sweeps, "residual": {"split": "tensor cores, exact BF16 slices",
                                                          "fp64": "FP64 pipe"}[res],
                          "ms": mms, "tflops": flops / (mms / 1e3) / 1e12,
                          "rel_err_vs_fp64": float(torch.linalg.norm(B - X64)) / ref})
        del X64
    line = {
        "metric": "batched_trsm_tflops", "value": flops / (ms / 1e3) / 1e12, "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded)",
        "config": {"workload": "batched_trsm_LLN_%s_%d_uneven" % (args.dtype, args.count), "count": args.count,
                   "n": "log-uniform [16, 1024]", "m": "uniform 1..128", "seed": 7, "flops": flops,
                   "nodes": items, "persistent_ctas": grid,
                   "tuning": {"cutoff": cutoff, "cols": cw} if tuned else "library defaults"},
        "one_launch_per_system": {"ms": loop_ms, "tflops": flops / (loop_ms / 1e3) / 1e12},
        "speedup_vs_one_launch_per_system": loop_ms / ms,
        "trace": {k: {"launches": v[0], "ms": v[1]} for k, v in trace.items()},
    }
    if mixed is not None:
        line["mixed_refined"] = mixed
    print(json.dumps(line), flush=True)
    plan.close()
    return 0


def run_error_table(args):
    """Float64 TRSM L/L/N at n x m with A graded to cond(A) in --conds (LAPACK
    dtrcon 1-norm estimate): for each cond, the plain FP64 solve (the FP64
    oracle of this table) and every mixed configuration (BF16 / FP16 slices,
    1-3 terms and 7 exact BF16 terms, 0-3 refinement sweeps).  One JSON line
    each: time, TFLOP/s, normwise relative error against the FP64 solution
    and backward error (double-double residual on 64 sampled columns)."""
    import numpy as np
    import torch

    import __graft_entry__ as graft

    pkg = graft.load_package()
    from nextla_gb300 import workloads

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n, m = args.n, args.m
    flops = float(n) * n * m
    rng = np.random.default_rng(1)
    B_h = np.asfortranarray(rng.uniform(-1.0, 1.0, (n, m)))
    B0 = torch.from_numpy(np.ascontiguousarray(B_h.T)).to(dev).T
    cols = torch.arange(0, m, max(1, m // 64), device=dev)

    def berr(A, X):
        Xs = X[:, cols].contiguous().T.contiguous().T
        Bs = B0[:, cols].contiguous().T.contiguous().T
        Rs = torch.empty_like(Xs.T).T
        pkg.residual_("L", "L", "N", 1.0, A, Xs, Bs, Rs, residual="dd")
        torch.cuda.synchronize(dev)
        an = float(torch.tril(A).abs().sum(dim=1).max())
        return float(Rs.abs().sum(dim=1).max() / (an * Xs.abs().sum(dim=1).max() * n * 2.0 ** -53))

    def timed(fn, A):
        X = torch.empty_like(B0.T).T
        X.copy_(B0)
        fn(A, X)  # warm-up (also sizes the workspace pools)
        X.copy_(B0)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn(A, X)
        e1.record()
        torch.cuda.synchronize(dev)
        pkg.device_status(X)
        return X, e0.elapsed_time(e1)

    for target in [float(c) for c in args.conds.split(",")]:
        A_h, c, cond = workloads.conditioned(n, target, seed=0)
        A = torch.from_numpy(np.ascontiguousarray(A_h.T)).to(dev).T
        del A_h
        Xref, pms = timed(lambda A_, X_: pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", A_, X_, native=True), A)
        ref_norm = float(torch.linalg.norm(Xref))
        base = {"n": n, "m": m, "cond_target": target, "cond1_dtrcon": cond, "diag_scale": c}
        print(json.dumps(dict(base, variant="plain_fp64", ms=pms, tflops=flops / pms / 1e9, rel_err=0.0,
                              backward_error=berr(A, Xref))), flush=True)
        configs = [("bf16", 7, 0)]
        if args.error_variants == "all":
            configs = [("bf16", t, sw) for t in (1, 2, 3) for sw in (0, 1, 2, 3)]
            configs += [("f16", t, sw) for t in (1, 2, 3) for sw in (0, 1, 2, 3)]
            configs += [("bf16", 7, sw) for sw in (0, 1)]
        for lowp, terms, sweeps in configs:
            fn = (lambda A_, X_, lowp=lowp, terms=terms, sweeps=sweeps:
                  pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A_, X_, lowp=lowp, split_terms=terms,
                                             sweeps=sweeps))
            X, ms = timed(fn, A)
            rel = float(torch.linalg.norm(X - Xref)) / ref_norm
            print(json.dumps(dict(base, variant="mixed", lowp=lowp, split_terms=terms, sweeps=sweeps, ms=ms,
                                  tflops=flops / ms / 1e9, rel_err=rel, backward_error=berr(A, X),
                                  finite=bool(torch.isfinite(X).all()))), flush=True)
            del X
        del A, Xref
    return 0


def run_callers(args):
    """The package's own callers on the GPU path, Float64, n = --n:
      getrf2_trsm   the recursive LU's triangular solve (src/lu.jl:277) at
                    the top split n1 = n/2: unit lower 8192 x 8192 with 8192
                    right-hand sides at n = 16384, on views of one array;
      lauum_trmm    every off-diagonal TRMM update of the blocked LAUUM
                    (src/lauum.jl:110 and :162), block size 512.
    One JSON line each: device time, flop rate (n1^2 (n - n1) and
    sum_i i b^2) and the relative error against scipy/numpy in FP64 on the
    host (the LU solve is checked on 64 sampled columns)."""
    import numpy as np
    import torch
    from scipy.linalg import solve_triangular

    import __graft_entry__ as graft

    pkg = graft.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n = args.n
    rng = np.random.default_rng(5)

    def timed(fn):
        fn()  # warm-up
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1)

    n1 = n // 2
    A_h = rng.standard_normal((n, n))
    A_h[:n1, :n1] = np.tril(A_h[:n1, :n1], -1) / np.sqrt(n1) + np.triu(A_h[:n1, :n1])
    A0 = torch.from_numpy(np.ascontiguousarray(A_h.T)).to(dev).T
    Ad = torch.empty_like(A0.T).T

    cols = np.arange(n1, n, max(1, (n - n1) // 64))
    L11 = np.tril(A_h[:n1, :n1], -1) + np.eye(n1)
    want = solve_triangular(L11, A_h[:n1, cols], lower=True, unit_diagonal=True)
    flops = float(n1) * n1 * (n - n1)
    copy_ms = timed(lambda: Ad.copy_(A0))
    for mixed in (False, True):
        def lu_step():
            Ad.copy_(A0)
            pkg.getrf2_trsm_(Ad, n1, mixed=mixed)

        ms = timed(lu_step) - copy_ms  # Ad holds the solved step afterwards
        got = Ad[:n1, torch.from_numpy(cols).to(dev)].cpu().numpy()
        print(json.dumps({"caller": "getrf2_trsm", "ref": "src/lu.jl:277", "n": n, "n1": n1, "dtype": "f64",
                          "form": "exact tensor-core updates" if mixed else "plain FP64", "ms": ms,
                          "tflops": flops / ms / 1e9,
                          "rel_err": float(np.linalg.norm(got - want) / np.linalg.norm(want))}), flush=True)
    del Ad, A0
    ib = 512
    for uplo in "UL":
        T = np.triu(rng.standard_normal((n, n))) if uplo == "U" else np.tril(rng.standard_normal((n, n)))
        T0 = torch.from_numpy(np.ascontiguousarray(T.T)).to(dev).T
        Td = torch.empty_like(T0.T).T

        i = (n // ib // 2) * ib  # one panel checked against numpy
        blk = T[i:i + ib, i:i + ib]
        want = T[:i, i:i + ib] @ blk.T if uplo == "U" else blk.T @ T[i:i + ib, :i]
        flops = float(sum(i * ib * ib for i in range(ib, n, ib)))
        copy_ms = timed(lambda: Td.copy_(T0))
        for mixed in (False, True):
            def lauum_updates():
                Td.copy_(T0)
                for k in range(ib, n, ib):
                    pkg.lauum_offdiag_trmm_(uplo, Td, k, min(ib, n - k), mixed=mixed)

            ms = timed(lauum_updates) - copy_ms  # Td holds the updated panels afterwards
            got = (Td[:i, i:i + ib] if uplo == "U" else Td[i:i + ib, :i]).cpu().numpy()
            print(json.dumps({"caller": "lauum_trmm_" + uplo, "ref": "src/lauum.jl:110" if uplo == "U" else
                              "src/lauum.jl:162", "n": n, "block": ib, "dtype": "f64",
                              "form": "exact tensor-core updates" if mixed else "plain FP64", "ms": ms,
                              "tflops": flops / ms / 1e9,
                              "rel_err_one_panel": float(np.linalg.norm(got - want) / np.linalg.norm(want))}),
                  flush=True)
        del Td, T0
    return 0


def run_sweep_plain(args):
    """Dtype-preserving TRSM and TRMM in Float32 and Float64 over all 8
    side/uplo/trans forms (trans N, T), alpha = 0.5, B n x n uniform[-1, 1],
    A built as in config 0 (seeded): one JSON line per case with the
    device time, n^3 flop rate and the relative error of 64 sampled columns
    against an FP64 (double-double residual for solves) check."""
    import itertools

    import numpy as np
    import torch

    import __graft_entry__ as graft

    pkg = graft.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    for n in [int(x) for x in args.sizes.split(",")]:
        rng = np.random.default_rng(n)
        Z = rng.standard_normal((n, n)) / np.sqrt(n)
        d = 2.0 + np.abs(rng.standard_normal(n))
        B_h = rng.uniform(-1.0, 1.0, (n, n))
        B64 = torch.from_numpy(np.ascontiguousarray(B_h.T)).to(dev).T
        for uplo in "LU":
            T = np.tril(Z, -1) if uplo == "L" else np.triu(Z, 1)
            T[np.diag_indices(n)] = d
            A64 = torch.from_numpy(np.ascontiguousarray(T.T)).to(dev).T
            del T
            for dtype, side, trans, func in itertools.product([torch.float32, torch.float64], "LR", "NT", "SM"):
                A = A64.to(dtype).T.contiguous().T
                B0 = B64.to(dtype).T.contiguous().T
                X = torch.empty_like(B0.T).T
                X.copy_(B0)
                pkg.unified_rectrxm_(side, uplo, trans, 0.5, func, A, X, native=True)  # warm-up
                X.copy_(B0)
                torch.cuda.synchronize(dev)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                pkg.unified_rectrxm_(side, uplo, trans, 0.5, func, A, X, native=True)
                e1.record()
                torch.cuda.synchronize(dev)
                ms = e0.elapsed_time(e1)
                # accuracy on sampled columns (rows for side R) in FP64
                idx = torch.arange(0, n, max(1, n // 64), device=dev)
                opA = (torch.tril(A64) if uplo == "L" else torch.triu(A64))
                opA = opA.T if trans == "T" else opA
                if side == "L":
                    Xs, Bs = X[:, idx].double(), B64[:, idx]
                    lhs = opA @ Xs if func == "S" else Xs
                    rhs = 0.5 * Bs if func == "S" else 0.5 * (opA @ Bs)
                else:
                    Xs, Bs = X[idx, :].double(), B64[idx, :]
                    lhs = Xs @ opA if func == "S" else Xs
                    rhs = 0.5 * Bs if func == "S" else 0.5 * (Bs @ opA)
                rel = float(torch.linalg.norm(lhs - rhs) / torch.linalg.norm(rhs))
                print(json.dumps({"n": n, "dtype": str(dtype).split(".")[-1], "func": func, "side": side,
                                  "uplo": uplo, "trans": trans, "ms": ms,
                                  "tflops": float(n) ** 3 / (ms / 1e3) / 1e12, "rel_check": rel}), flush=True)
                del A, B0, X
            del A64
        del B64
    return 0


def run_config3(args):
    """(1) TRMM side R, uplo U, trans T, n = 12288, B 12288 x 12288 Float64,
    updates from 3-term BF16 splits (FP64 diagonal blocks), against the plain
    FP64 TRMM of the same inputs; (2) TRSM L/L/N with Float16 A and B,
    n = 8192, m = 4096 (A: diagonal 2+|N(0,1)|, off-diagonals N(0,1)/sqrt(n)),
    Float16 updates on tensor cores with FP32 accumulation, against an FP64
    solve of the same (Float16-rounded) inputs."""
    import numpy as np
    import torch

    import __graft_entry__ as graft

    pkg = graft.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1)

    n = 12288
    rng = np.random.default_rng(3)
    T = np.triu(rng.standard_normal((n, n)) / np.sqrt(n), 1)
    T[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
    A = torch.from_numpy(np.ascontiguousarray(T.T)).to(dev).T
    del T
    B0 = torch.from_numpy(np.ascontiguousarray(rng.uniform(-1, 1, (n, n)).T)).to(dev).T
    ref = torch.empty_like(B0.T).T

    def plain():
        ref.copy_(B0)
        pkg.unified_rectrxm_("R", "U", "T", 1.0, "M", A, ref, native=True)

    pms = timed(plain)
    X = torch.empty_like(B0.T).T

    def mixed():
        X.copy_(B0)
        pkg.unified_rectrxm_mixed_("R", "U", "T", 1.0, "M", A, X, lowp="bf16", split_terms=3)

    ms = timed(mixed)
    rel = float(torch.linalg.norm(X - ref) / torch.linalg.norm(ref))
    flops = float(n) ** 3
    print(json.dumps({"case": "trmm_RUT_f64_mixed_bf16x3_n12288", "ms": ms, "tflops": flops / ms / 1e9,
                      "plain_fp64_ms": pms, "plain_fp64_tflops": flops / pms / 1e9, "rel_err_vs_fp64": rel}),
          flush=True)
    del A, B0, ref, X

    n, m = 8192, 4096
    rng = np.random.default_rng(4)
    T = np.tril(rng.standard_normal((n, n)) / np.sqrt(n), -1)
    T[np.diag_indices(n)] = 2.0 + np.abs(rng.standard_normal(n))
    A16 = torch.from_numpy(np.ascontiguousarray(T.T)).to(dev).T.half().T.contiguous().T
    del T
    B16 = torch.from_numpy(np.ascontiguousarray(rng.uniform(-1, 1, (n, m)).T)).to(dev).T.half().T.contiguous().T
    X16 = torch.empty_like(B16.T).T

    def f16():
        X16.copy_(B16)
        pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", A16, X16, native=True)

    from nextla_gb300 import _lib

    ms = timed(f16)
    _lib.trace_enable(True)
    f16()
    torch.cuda.synchronize(dev)
    _lib.trace_enable(False)
    trace = {k: {"launches": v[0], "ms": v[1]} for k, v in _lib.trace_summary().items()}
    A64 = A16.double().T.contiguous().T
    X64 = B16.double().T.contiguous().T
    pkg.unified_rectrxm_("L", "L", "N", 1.0, "S", A64, X64, native=True)
    torch.cuda.synchronize(dev)
    rel = float(torch.linalg.norm(X16.double() - X64) / torch.linalg.norm(X64))
    print(json.dumps({"case": "trsm_LLN_f16_n8192_m4096", "ms": ms, "tflops": float(n) * n * m / ms / 1e9,
                      "rel_err_vs_fp64": rel, "unit_roundoff_f16": 2.0 ** -11, "trace": trace}), flush=True)
    return 0


def run_kernel_case(args):
    """Single launches of one kernel on an s x s case (s = --case-size),
    sized so that operands exceed L2 but the device holds a few GB at most:
      exact  one exact slice-product update, C (s x s) -= A (s x s) B (s x s),
             7 BF16 slices per operand (--case-shape M,N,K for C (M x N) -=
             A (M x K) B (K x N));
      fast   the same with 3 BF16 slices (FP32 accumulation);
      leaf   one FP64 diagonal-block solve of order 128 with 8 s right-hand
             sides (--case-shape n,m for order n with m right-hand sides);
      pair   one exact mixed solve (L/L/N, 7 BF16 slices, 0 sweeps) of order
             s with 4 s right-hand sides, whose 128-row nodes each run one
             leaf_pair_kernel launch (s / 128 per solve);
      dfma   one FP64 update on CUDA cores, s x s x s."""
    import torch

    import __graft_entry__ as graft

    pkg = graft.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    g = torch.Generator(device=dev).manual_seed(0)
    s = args.case_size

    def cm(r, c):
        return torch.randn(c, r, generator=g, device=dev, dtype=torch.float64).T

    times = []
    for _ in range(args.case_reps):
        if args.kernel_case in ("exact", "fast"):
            M, N, K = (int(x) for x in args.case_shape.split(",")) if args.case_shape else (s, s, s)
            A, B, C = cm(M, K), cm(K, N), cm(M, N)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            pkg.matmul_mixed_(C, A, B, -1.0, split_terms=7 if args.kernel_case == "exact" else 3)
        elif args.kernel_case == "leaf":
            n, mr = (int(x) for x in args.case_shape.split(",")) if args.case_shape else (128, 8 * s)
            A = cm(n, n).tril_() + 4 * torch.eye(n, device=dev, dtype=torch.float64)
            A = A.T.contiguous().T
            B = cm(n, mr)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            pkg.LeftLowerTRSM_(A, B)
        elif args.kernel_case == "pair":
            A = (cm(s, s) / math.sqrt(s)).tril_(-1)
            A.diagonal().copy_(2.0 + torch.randn(s, generator=g, device=dev, dtype=torch.float64).abs())
            B = torch.rand(4 * s, s, generator=g, device=dev, dtype=torch.float64).T * 2.0 - 1.0
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            pkg.unified_rectrxm_mixed_("L", "L", "N", 1.0, "S", A, B, split_terms=7, sweeps=0)
        else:
            A, B, C = cm(s, s), cm(s, s), cm(s, s)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            pkg.GEMM_SUB_(C, A, B)
        pkg.device_status()
        times.append((time.perf_counter() - t0) * 1e3)
    print(json.dumps({"kernel_case": args.kernel_case, "size": s, "shape": args.case_shape or None,
                      "host_ms": times}), flush=True)
    return 0


def staged_a_elems(n, levels, cutoff):
    """Elements of A the host-buffer call copies in: the diagonal blocks where
    its staged walk stops and the off-diagonal blocks of the triangle above
    them."""
    if levels <= 0 or n <= cutoff:
        return n * n
    p = 1
    while p * 2 <= n:
        p *= 2
    mid = n // 2 if p == n else p
    return staged_a_elems(mid, levels - 1, cutoff) + mid * (n - mid) + staged_a_elems(n - mid, levels - 1, cutoff)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.kernel_case:
        return run_kernel_case(args)
    if args.cpu_table:
        return run_cpu_table(args)
    if args.sweep_plain:
        return run_sweep_plain(args)
    if args.callers:
        return run_callers(args)
    if args.config3:
        return run_config3(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.error_table:
        return run_error_table(args)

    import numpy as np
    import torch

    import __graft_entry__ as graft

    world, rank, local = rank_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    pkg = graft.load_package()
    L = pkg.load_library()
    from nextla_gb300 import _lib

    n, m = args.n, args.m
    A_h, B_h = make_inputs(n, m)
    flops = float(n) * n * m
    # Column-major device copies (tensor of shape (n, m) with strides (1, n)).
    A = torch.from_numpy(np.ascontiguousarray(A_h.T)).to(dev).T
    B0 = torch.from_numpy(np.ascontiguousarray(B_h.T)).to(dev).T
    B = torch.empty_like(B0.T).T
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    import ctypes

    opts = _lib.MixedOpts({"bf16": _lib.NLA_LOWP_BF16, "f16": _lib.NLA_LOWP_F16}[args.lowp], args.terms,
                          args.sweeps, {"split": _lib.NLA_RESIDUAL_SPLIT, "fp64": _lib.NLA_RESIDUAL_FP64}[args.residual],
                          args.cutoff, None)

    def solve_plain(Ad, Bd):
        _lib.check(L.nla_trxm(b"L", b"L", b"N", 1.0, b"S", _lib.NLA_F64, n, m, Ad.data_ptr(), n, Bd.data_ptr(), n,
                              sptr))

    def solve_mixed(Ad, Bd):
        _lib.check(L.nla_trxm_mixed(b"L", b"L", b"N", 1.0, b"S", n, m, Ad.data_ptr(), n, Bd.data_ptr(), n,
                                    ctypes.byref(opts), sptr))

    solve_fn = solve_mixed if args.variant == "mixed" else solve_plain

    def solve(Bd):
        solve_fn(A, Bd)

    def step():
        B.copy_(B0)
        solve(B)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(args.warmup):
        step()
    barrier()

    sampler = ClockSampler(local)
    sampler.start()
    _lib.trace_enable(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    _lib.trace_enable(False)
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    ms_per_step = ms / args.steps
    value = job_tflops(world, args.steps * flops, ms)
    trace = _lib.trace_summary()

    # Accuracy of the last solution on a sample of columns: backward error
    # ||A X - B||_inf / (||A||_inf ||X||_inf n u), residual accumulated in
    # double-double (the library's NLA_RESIDUAL_DD mode).
    cols = torch.arange(0, m, max(1, m // 64), device=dev)

    def backward_error(Xfull):
        Xs_ = Xfull[:, cols].contiguous().T.contiguous().T
        Bs_ = B0[:, cols].contiguous().T.contiguous().T
        Rs_ = torch.empty_like(Xs_.T).T
        pkg.residual_("L", "L", "N", 1.0, A, Xs_, Bs_, Rs_, residual="dd")
        torch.cuda.synchronize(dev)
        an = float(torch.tril(A).abs().sum(dim=1).max())
        rn = float(Rs_.abs().sum(dim=1).max())
        xn = float(Xs_.abs().sum(dim=1).max())
        return rn / (an * xn * n * 2.0 ** -53), {"r_inf": rn, "a_inf": an, "x_inf": xn}

    # End to end through the C ABI with host buffers: the host-buffer entry
    # point copies A's triangle and B in and X out in blocks pipelined with
    # the recursion.
    # Page-locked host buffers from the library (cudaHostAlloc), as a caller
    # of the host-buffer entry point would use.
    A_pin = _lib.host_empty(n * n, torch.float64).view(n, n)
    A_pin.copy_(torch.from_numpy(np.ascontiguousarray(A_h.T)))
    B_pin = _lib.host_empty(m * n, torch.float64).view(m, n)
    B_pin.copy_(torch.from_numpy(np.ascontiguousarray(B_h.T)))
    X_pin = _lib.host_empty(m * n, torch.float64).view(m, n)
    Ae = torch.empty_like(A.T)
    Be = torch.empty_like(B0.T)

    def e2e_step():
        if args.variant == "mixed":
            _lib.check(L.nla_trxm_mixed_host(b"L", b"L", b"N", 1.0, b"S", n, m, A_pin.data_ptr(), n,
                                             B_pin.data_ptr(), n, X_pin.data_ptr(), n, Ae.data_ptr(), n,
                                             Be.data_ptr(), n, ctypes.byref(opts), args.host_levels, sptr))
        else:
            _lib.check(L.nla_trxm_host(b"L", b"L", b"N", 1.0, b"S", _lib.NLA_F64, n, m, A_pin.data_ptr(), n,
                                       B_pin.data_ptr(), n, X_pin.data_ptr(), n, Ae.data_ptr(), n, Be.data_ptr(),
                                       n, args.host_levels, sptr))

    def sequential_step():
        Ae.copy_(A_pin, non_blocking=True)
        Be.copy_(B_pin, non_blocking=True)
        solve_fn(Ae.T, Be.T)
        X_pin.copy_(Be, non_blocking=True)

    # Each end-to-end step ends when its result is back on the host (a
    # synchronize, as a caller reading X must); the median step is reported.
    def timed_steps(fn, count):
        fn()
        barrier()
        times = []
        for _ in range(count):
            t0 = time.perf_counter()
            fn()
            barrier()
            times.append(time.perf_counter() - t0)
        return times

    e2e_steps = E2E_STEPS
    e2e_times = timed_steps(e2e_step, e2e_steps)
    # The credited figure is the mean step (slowest rank); median and max are
    # reported beside it.
    e2e_s = max_over_ranks(statistics.mean(e2e_times) * 1e3, world, dev) / 1e3
    e2e_value = job_tflops(world, flops, e2e_s * 1e3)
    host_levels = args.host_levels if args.host_levels > 0 else int(os.environ.get("NLA_HOST_LEVELS", "3"))
    host_cutoff = args.cutoff if args.cutoff > 0 else (64 if args.variant == "mixed" else 256)
    # The host-buffer result against the device-resident solve of the timed loop.
    e2e_same = bool(torch.equal(X_pin, B.T.cpu()))
    # The same with copy-in, solve and copy-out one after another, and one
    # more such step with device events between its phases: where the time
    # goes without the pipelining.
    seq_times = timed_steps(sequential_step, e2e_steps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    Ae.copy_(A_pin, non_blocking=True)
    Be.copy_(B_pin, non_blocking=True)
    ev[1].record(stream)
    solve_fn(Ae.T, Be.T)
    ev[2].record(stream)
    X_pin.copy_(Be, non_blocking=True)
    ev[3].record(stream)
    barrier()
    e2e_phases = {"h2d_ms": ev[0].elapsed_time(ev[1]), "solve_ms": ev[1].elapsed_time(ev[2]),
                  "d2h_ms": ev[2].elapsed_time(ev[3]),
                  "sequential_step_ms": round(statistics.median(seq_times) * 1e3, 2)}

    berr, berr_parts = backward_error(B)
    plain = None
    if args.variant == "mixed" and not args.no_plain:
        # The plain FP64 path on the same inputs: one warm-up solve, then
        # PLAIN_STEPS timed solves (each restoring B first), the slowest
        # rank's time, the whole-job rate, as for `value`.
        Bp = torch.empty_like(B0.T).T
        Bp.copy_(B0)
        solve_plain(A, Bp)  # warm-up of the plain path's kernels
        barrier()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(PLAIN_STEPS):
            Bp.copy_(B0)
            solve_plain(A, Bp)
        p1.record(stream)
        barrier()
        pms = max_over_ranks(p0.elapsed_time(p1), world, dev)
        pb, pparts = backward_error(Bp)
        plain = {"tflops": job_tflops(world, PLAIN_STEPS * flops, pms), "ms_per_step": pms / PLAIN_STEPS,
                 "backward_error": pb, "norms": pparts, "steps": PLAIN_STEPS}
        del Bp

    # Roofline of the dominant kernel class.
    pk, pk_kind = peaks()
    pipes = _lib.measure_pipes(sptr)
    dom = max(trace.items(), key=lambda kv: kv[1][1]) if trace else None
    roofline = None
    gpu_launches = sum(v[0] for v in trace.values())
    if dom:
        name, (launches, kms, kflops, kbytes) = dom
        achieved = kflops / (kms / 1e3) / 1e12
        share = kms / sum(v[1] for v in trace.values())
        # The committed DRAM capture covers the exact 7-slice updates of the
        # 16384 x 16384 solve only.
        exact_headline = (args.variant == "mixed" and args.terms == 7 and args.n == 16384 and args.m == 16384)
        if name == "gemm_umma":
            peak = float(pk.get("bf16_tflops_sustained", pk.get("bf16_tflops")))
            roofline = {"kernel": "umma_gemm/umma_exact (tcgen05 BF16 slice products)", "bound": "tensor",
                        "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                        "traffic": TRAFFIC_BYTES_PER_LAUNCH if exact_headline else None,
                        "traffic_source": TRAFFIC_SOURCE if exact_headline else None,
                        "launches": launches, "share": share,
                        "peak_source": "bf16_tflops_sustained of %s MEASURED_PEAKS.json" % pk_kind}
        else:
            # The plain FP64 path runs on the DFMA pipe; no tensor or HBM peak applies.
            dfma = pipes["dfma"]
            roofline = {"kernel": name, "bound": "fp64", "achieved": achieved, "peak": dfma,
                        "unit": "TFLOP/s", "frac": achieved / dfma, "traffic": None,
                        "launches": launches, "share": share,
                        "peak_source": "DFMA probe measured live (nla_measure_pipes)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = args.cpu_sample or 128 * threads
        v, dt = cpu_baseline(A_h, B_h, sample, threads)
        cpu = {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": "port",
               "sample": "%d of %d right-hand sides, full %dx%d A, %.1f s" % (sample, m, n, n, dt)}

    if rank == 0:
        line = {
            "metric": "trsm_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": {"workload": "trsm_LLN_f64_n%d_m%d" % (n, m), "n": n, "m": m, "side": "L",
                       "uplo": "L", "trans": "N", "alpha": 1.0, "variant": args.variant,
                       "mixed": ({"lowp": args.lowp, "split_terms": args.terms, "sweeps": args.sweeps,
                                  "residual": args.residual, "cutoff": args.cutoff or "default"}
                                 if args.variant == "mixed" else None),
                       "l2": "inputs larger than L2", "parallelism": "replicas" if world > 1 else "single"},
            "accuracy": {"backward_error": berr, "norms": berr_parts,
                         "definition": "||AX-B||_inf/(||A||_inf ||X||_inf n u), 64 sampled columns, "
                                       "residual in double-double"},
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["tflops"]) if plain else None,
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "phases_ms": e2e_phases,
                    "statistic": "mean of %d synchronised steps" % len(e2e_times),
                    "step_ms_mean": round(statistics.mean(e2e_times) * 1e3, 2),
                    "step_ms_median": round(statistics.median(e2e_times) * 1e3, 2),
                    "step_ms_max": round(max(e2e_times) * 1e3, 2),
                    "step_ms": [round(t * 1e3, 2) for t in e2e_times],
                    "h2d_bytes_per_step": int(8 * staged_a_elems(n, host_levels, host_cutoff) + B_h.nbytes),
                    "d2h_bytes_per_step": int(B_h.nbytes), "host_levels": host_levels,
                    "matches_device_result": e2e_same},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": gpu_launches,
            "trace": {k: {"launches": v[0], "ms": v[1], "tflops": v[2] / max(v[1], 1e-9) / 1e9}
                      for k, v in trace.items()},
            "pipes_tflops": pipes,
            "peaks": pk_kind,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
