"""bench.py's reference arm on the CPU: one JSON line with the contract's keys.

The reference arm times the reference's CPU path (the compiled reference
where it builds, else the oracle port) on the host cores; it needs no GPU.
A small point count keeps the test short (the grid stays M = 2688).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--n", "2048", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(rows) == 1, r.stdout[-2000:]
    return json.loads(rows[0])


def test_reference_arm_line_has_the_contract_keys(line):
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["unit"] == "evals/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 0
    assert abs(line["ms_per_step"] - 1e3 / line["value"]) < 1e-6 * line["ms_per_step"]


def test_reference_arm_baseline_and_e2e(line):
    cb, e2e = line["cpu_baseline"], line["e2e"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"]
    assert e2e == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}
    assert line["config"]["N_sources"] == 2048 and line["config"]["M"] == 2688
