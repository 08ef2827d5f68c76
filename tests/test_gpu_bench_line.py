"""bench.py's own arm on the GPU, on a reduced workload (4 shots, 60 time
steps): one JSON line with the benchmark contract's fields and the
reporting objects (roofline, e2e with the batch plan, plain path, clocks,
kernel launches, the tuner's choices)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_line_fields():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--shots", "4", "--nt", "60", "--steps", "2",
                        "--warmup", "3", "--no-cpu"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "e2e", "plain", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["metric"] == "shot-gradients/s" and d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 2
    roof = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in roof, k
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and 0 < roof["frac"] and roof["achieved"] > 0
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert e2e["batch_plan"]["time_stepping"] in ("two-step", "single", "single-fused")
    assert e2e["batch_plan"]["launch"][0] in ("graph", "direct", "undecided")
    assert d["plain"]["value"] > 0 and d["gpu_launches"] > 0
    c = d["config"]
    assert "workload" in c and c["time_stepping"]["form"] in ("two-step", "single", "single-fused")
    assert c["launch"]["form"] in ("graph", "direct", "undecided")
    assert c["shots_per_gpu"] == 4
    # clocks are sampled during the timed region; this one is a few tens of
    # milliseconds, shorter than the sampling interval, so it may hold none
    if d["clocks"] is not None:
        assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
