"""bench.py's multi-rank path on CPU: two gloo ranks (world size 2).

The path shards nothing: each rank solves its own replica, so the only
collectives are the barriers and the max-over-ranks reduction of the timed
region.  Checked here:
  - every rank gets the slowest rank's time;
  - the whole-job rate counts all ranks' work in that time;
  - the speed-up over the plain FP64 path compares two whole-job rates, so
    it does not grow with the number of ranks;
  - under torchrun, the reference arm runs on rank 0 only.
"""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        dist.barrier()
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, torch.device("cpu"))
        rate = bench.job_tflops(world, 2e12, ms)
        # The plain comparison goes through the same reduction and rate: its
        # ranks take 400 and 200 ms for 3 steps of the same work.
        plain_ms = bench.max_over_ranks(400.0 - 200.0 * rank, world, torch.device("cpu"))
        plain_rate = bench.job_tflops(world, 3 * 2e12, plain_ms)
        dist.barrier()
        with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
            json.dump({"ms": ms, "rate": rate, "speedup": rate / plain_rate}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_over_ranks(tmp_path):
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    for rank in range(world):
        got = json.load(open(tmp_path / ("rank%d.json" % rank)))
        assert got["ms"] == 20.0  # the slower rank's 20 ms, on both ranks
        assert got["rate"] == pytest.approx(2 * 2e12 / 0.020 / 1e12)  # 200 TFLOP/s of whole-job work
        # 20 ms per step against 400 / 3 ms per plain step: 6.67x, whatever the world size.
        assert got["speedup"] == pytest.approx((400.0 / 3) / 20.0)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(12.5, 1, None) == 12.5
    assert bench.job_tflops(1, 1e12, 1000.0) == pytest.approx(1.0)


def test_reference_arm_other_ranks_exit_quietly(oracle):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--n", "256", "--m", "64", "--cpu-sample", "16"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
