"""bench.py's CPU reference arm: one JSON line with the contract's keys, the
same metric, unit and direction as the GPU arm, a cpu_baseline describing the
run, and complete measured work: the steps together build the whole basis and
apply one whole matvec, the time they report fits in the run, and the
modelled per-solve value says that it is extrapolated. The 24-site chain
keeps this quick; the 6x6 config's line is checked for its config."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    t = __import__("time").perf_counter()
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "chain24", "--steps", "4",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    wall = __import__("time").perf_counter() - t
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "s" and line["higher_is_better"] is False
    cb = line["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"} and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["value"] == line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["steps"] == 4 and line["warmup"] == 1 and line["n_gpus"] == 1
    meas = line["measured"]
    assert meas["D"] == bench.CHAIN24_D and len(meas["steps_s"]) == 4
    assert line["extrapolated"] is True
    assert abs(line["ms_per_step"] * 4 / 1e3 - meas["total_s"]) < 1e-9
    assert line["ms_per_step"] * 4 / 1e3 <= wall  # the reported work fits in the run
    assert line["value"] == meas["basis_build_s"] + bench.SOLVE_MATVECS["chain24"] * meas["matvec_s"]


def test_reference_config_matches_gpu_arm():
    sys.path.insert(0, ROOT)
    import bench
    assert bench._reference_config("square6", 1) == bench.workload_config(
        "square6", "fp64", bench.SQUARE6_D, bench.SQUARE6_ELEMENTS, bench.SQUARE6_STREAM_BYTES, 1)
