"""bench.py's JSON contract on a small fragment (GPU): one line with the
metric, throughput, roofline, e2e and clock fields, and an accuracy check
against the FP64 kernel that passes the 1e-7 bar."""
import json
import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def test_bench_json_line_small_fragment():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--nocc", "8", "--nvirt", "256",
           "--nba", "512", "--steps", "2", "--warmup", "1", "--cpu-seconds", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "roofline",
              "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "TFLOP/s" and d["steps"] == 2
    assert d["config"]["workload"]
    rf = d["roofline"]
    assert rf["bound"] == "tensor" and 0 < rf["frac"] < 1.2 and rf["achieved"] > 0, rf
    assert d["e2e"]["h2d_bytes_per_step"] == 8 * (512 * 256 * 8 + 8 + 256)
    assert d["gpu_launches"] >= 2
    assert d["accuracy"]["within_1e-7"]
    assert d["plain_fp64"]["frac_of_fp64_peak"] > 0.3
