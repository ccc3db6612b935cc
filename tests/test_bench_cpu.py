"""bench.py on the CPU: the reference arm's JSON line (the oracle on the host cores, a bounded sample of
the default workload) and the first-come-first-served latency model of the serving comparison."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def test_fcfs_latency_model():
    import bench

    # arrivals at 1, 2, 3 s; services 0.5, 2, 0.1 s: the third waits for the second
    lat = bench.fcfs_latency_ms([1.0, 1.0, 1.0], [0.5, 2.0, 0.1])
    assert lat == pytest.approx([500.0, 2000.0, 1100.0])


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_batch_sort_passes_rule():
    import bench

    assert bench.batch_sort_passes(24, 2) == (24, 3)        # a frame: 1 tag bit over 24 dropped, 3 passes
    assert bench.batch_sort_passes(24, 1) == (24, 3)
    assert bench.batch_sort_passes(24, 2, True) == (24, 3)  # one more bit for empty slots, dropped too
    assert bench.batch_sort_passes(20, 2) == (21, 3)
    assert bench.batch_sort_passes(27, 300) == (31, 4)      # 9 tag bits: 36 -> 31 bits, 4 passes
    assert bench.batch_sort_passes(24, 300) == (31, 4)
    assert bench.batch_sort_passes(17, 300) == (24, 3)      # 26 bits: 2 leftover bits dropped
