"""bench.py's reference arm (the CPU path timed on the host cores): its JSON line on CPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"]


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_reference_arm_line():
    line = _run("--steps", "1", "--warmup", "0")
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "TFLOP/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    rec = line["config"]["reference_binary_recorded"]
    assert rec["cores"] == 1 and rec["ccsd_s"] > 3600 and rec["ccsd_iterations"] == 10


def test_reference_arm_reports_unavailable_where_the_cpu_path_cannot_run():
    line = _run("--workload", "c3", "--steps", "1", "--warmup", "0")
    assert line["impl"] == "reference" and "unavailable" in line
