"""bench.py's reference arm (the oracle timed on host cores) keeps the JSON contract the
benchmark harness reads; it runs on the CPU, here on a small sample."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def run_reference(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-sample", "6"], capture_output=True, text=True, timeout=300,
                       cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_reference_arm_line():
    lines = [l for l in run_reference().splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "DOF/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("poisson3d_kuhn_128^3")


def test_reference_arm_other_ranks_print_nothing():
    assert run_reference({"RANK": "1"}).strip() == ""
