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
    line = _run("--workload", "c2", "--steps", "1", "--warmup", "0")
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "TFLOP/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    rec = line["config"]["reference_binary_recorded"]
    assert rec["cores"] == 1 and rec["ccsd_s"] > 3600 and rec["ccsd_iterations"] == 10


def test_reference_arm_samples_triples_tuples_at_the_default_workload():
    """no=32/nv=320: the CPU CCSD iteration needs <ab|ef> (84 GB); each step is one (T)
    tuple term of the oracle instead, with the same metric and unit as the GPU arm."""
    line = _run("--steps", "1", "--warmup", "0")
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "TFLOP/s"
    assert line["config"]["workload"] == "ccsd_t_no32_nv320_seed2"
    assert "tuple" in line["config"]["step"] and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["d2h_bytes_per_step"] == 0
