"""bench.py's reference arm on the host cores: one JSON line with the keys
the benchmark contract names (a small workload; no GPU involved)."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line(oracle):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--n", "256", "--m", "64", "--cpu-sample", "16"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "trsm_tflops" and line["unit"] == "TFLOP/s" and line["higher_is_better"] is True
    assert line["value"] > 0
    assert line["config"]["workload"] == "trsm_LLN_f64_n256_m64"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_traffic_figure_matches_its_profile():
    """roofline.traffic is the figure of one committed ncu capture: the
    constant in bench.py, the capture's summary under profiles/ and the
    commit stamped beside it agree."""
    import re

    src = open(os.path.join(ROOT, "bench.py")).read()
    value = float(re.search(r"^TRAFFIC_BYTES_PER_LAUNCH = ([0-9.e+]+)$", src, re.M).group(1))
    commit = re.search(r"at commit ([0-9a-f]{7,40})", src).group(1)
    summary = open(os.path.join(ROOT, "profiles", "umma_exact_kernel_n16384_dram.md")).read()
    assert "traffic_bytes_per_launch: %d" % round(value) in summary
    assert "Commit %s" % commit in summary
