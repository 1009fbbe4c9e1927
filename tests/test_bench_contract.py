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
    # the sample it ran is the workload it names, with the GPU arm's config keys
    assert d["config"]["workload"] == "poisson3d_kuhn_6^3_sigma2"
    assert set(d["config"]) == {"workload", "dofs", "free_dofs", "elements", "nnz", "precision", "tolerance", "l2"}
    assert d["config"]["dofs"] == 7 ** 3 and d["config"]["elements"] == 6 * 6 ** 3
    assert d["config"]["precision"] == "mixed" and d["dtype"] == "f64+f32"


def test_reference_arm_other_ranks_print_nothing():
    assert run_reference({"RANK": "1"}).strip() == ""
