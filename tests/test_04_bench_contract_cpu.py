"""bench.py's CPU reference arm: one JSON line with the contract's keys, the
same metric, unit, direction and workload config as the GPU arm, and a
cpu_baseline describing the run (a short sample budget keeps this quick)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--cpu-budget", "0.5"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["config"] == bench.workload_config("square6", "fp64", bench.SQUARE6_D, bench.SQUARE6_ELEMENTS,
                                                   bench.SQUARE6_STREAM_BYTES, 1)
    cb = line["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"} and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["value"] == line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["steps"] == 1 and line["warmup"] == 0 and line["n_gpus"] == 1
