"""bench.py pieces that need no GPU: the reference arm's JSON line (the
CPU restatement of RIMP2.F90's path on a bounded sample of pairs), the
workload generators and the effective-FLOP count."""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT


def test_reference_arm_json_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "TFLOP/s" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_workload_generators_and_flop_count():
    sys.path.insert(0, ROOT)
    import bench
    s1, s2 = bench.batch_shapes(), bench.batch_shapes()
    assert s1 == s2 and len(s1) == 256
    assert all(8 <= o <= 64 and 64 <= v <= 512 and 256 <= b <= 2048 for o, v, b in s1)
    ao = bench.ao_shapes(64)
    assert all(128 <= nb <= 768 and nba == 3 * nb and no == nb // 10 and nv == nb - nb // 10
               for nb, nba, no, nv in ao)
    # 2 NBA (nocc nvirt)^2 at the large fragment
    assert bench.eff_flop(128, 1024, 4096) == 2.0 * 4096 * (128 * 1024) ** 2
    assert abs(bench.eff_flop(128, 1024, 4096) - 1.407e14) / 1.407e14 < 1e-3


def test_performed_tiles_match_enumeration():
    """The performed-work count of both energy kernels against an explicit
    enumeration of their work items."""
    sys.path.insert(0, ROOT)
    import bench
    for nocc in (1, 2, 5, 8, 33, 128):
        for nvirt in (1, 96, 128, 300, 1024):
            nt = (nvirt + 127) // 128
            tps = [(a, b) for b in range(nt) for a in range(b + 1)]
            one = sum(1 if (i == j or a == b) else 2
                      for j in range(nocc) for i in range(j + 1) for a, b in tps)
            pair = sum(2 * (1 if (a == b or i0 == j) else 2)
                       for j in range(nocc) for i0 in range(0, j + 1, 2) for a, b in tps)
            assert bench.performed_tiles(nocc, nvirt, False) == one
            assert bench.performed_tiles(nocc, nvirt, True) == pair
