"""bench.py's CPU-side pieces: the reference arm's JSON line (the oracle port on the host
cores, a small workload here) carries the keys the measurement contract names, and the
roofline helper's arithmetic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--cells", "8",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "cell-steps/s" and d["metric"] == bench.METRIC
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cells = bench.make_workload(seed=1000, ncells=8)
    assert {k: d["config"][k] for k in ("workload", "cells", "vertices", "triangles")} == bench.workload_config(cells)


def test_lu_roofline_arithmetic():
    r = bench.lu_roofline(200.0, 512)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert abs(r["frac"] - 200.0 / r["peak"]) < 1e-3 and "K = 512" in r["note"]
    assert bench.lu_roofline(None)["frac"] is None
    m = bench.lu_roofline(250.0, 512, tf32_peak=1000.0)
    assert m["peak"] == 1000.0 and m["frac"] == 0.25 and "measured TF32" in m["peak_source"]
