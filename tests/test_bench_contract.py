"""The JSON line of `bench.py --impl reference` (the CPU arm: the oracle's
restatement of the reference's step on the host cores), checked on the CPU:
one line of strict JSON with the keys and units the GPU arm reports, the
same metric string, and an end-to-end entry without host copies."""

import json
import math
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def line():
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl",
         "reference", "--steps", "3", "--warmup", "3"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert lines, "no output"
    return json.loads(lines[-1])


def test_reference_line_keys(line):
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps",
                "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline",
                "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "MLUPS"
    assert line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 3
    assert math.isfinite(line["value"]) and line["value"] > 0
    assert "workload" in line["config"]


def test_reference_line_matches_gpu_metric(line):
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.pop(0)
    assert line["metric"] == bench.METRIC


def test_reference_line_baseline_and_e2e(line):
    cb = line["cpu_baseline"]
    for key in ("value", "unit", "cores", "kind", "sample"):
        assert key in cb, key
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
