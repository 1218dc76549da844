"""bench.py's reference arm (the CPU port of the path, timed on the host's
cores) on a small workload: one JSON line with the keys the benchmark contract
names, a positive rate, and host-only end-to-end figures."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "32", "--directions",
           "64", "--cpu-sample", "8", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "8 of the 64" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["N"] == 32 and d["config"]["directions"] == 64
    # the line reports what it timed: value = the sample's directions / the measured step time
    assert d["directions_per_step"] == 8
    assert abs(d["value"] - 8 / (d["ms_per_step"] / 1e3)) <= 1e-9 * d["value"]
    assert d["full_step_extrapolated"]["value"] > 0
    # and the same config dict as the GPU arm
    import argparse

    sys.path.insert(0, ROOT)
    import bench

    ns = argparse.Namespace(size=32, directions=64, batch=2000, precision="f32")
    assert d["config"] == bench.bench_config(ns, 1)
