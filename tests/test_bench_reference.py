"""bench.py --impl reference (the reference's algorithm, timed on the host
cores through the CPU oracle) prints one JSON line with the fields the bench
contract asks of that arm. Runs on the CPU, with two worker threads."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# bench.py as a script, with os.cpu_count() pinned to 2 so that the test
# stays small on machines with many cores
WRAPPER = (
    "import os, runpy, sys; os.cpu_count = lambda: 2; "
    "sys.argv = ['bench.py'] + sys.argv[1:]; "
    "runpy.run_path('bench.py', run_name='__main__')"
)


def reference_line(*args):
    out = subprocess.run([sys.executable, "-c", WRAPPER, "--impl", "reference", *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def check_contract(line, metric, unit):
    assert line["impl"] == "reference"
    assert line["metric"] == metric and line["unit"] == unit
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["data"] == "synthetic"
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["unit"] == unit and cb["cores"] == 2 and cb["kind"] == "port"
    assert cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == unit
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


@pytest.mark.timeout(900)
def test_reference_arm_frame():
    line = reference_line("--steps", "1", "--warmup", "0")
    check_contract(line, "Mfrag/s", "Mfrag/s")


@pytest.mark.timeout(900)
def test_reference_arm_batch():
    line = reference_line("--workload", "batch", "--scenes", "4", "--steps", "1", "--warmup", "0")
    check_contract(line, "scenes/s", "scenes/s")
    assert line["config"]["scenes"] == 4
