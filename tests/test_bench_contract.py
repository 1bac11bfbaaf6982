"""The reference arm of bench.py on a tiny case, on the CPU: one JSON line with the metric, the
CPU port's own baseline description and an end-to-end figure with no host-device traffic; under
a multi-rank launch only rank 0 runs and prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--scale", "0.05", "--nsteps", "8", "--cpu-sample", "4", "--cpu-procs", "2",
        "--steps", "1", "--warmup", "1"]


def _run(extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], capture_output=True, text=True,
                          env=env, timeout=300, cwd=ROOT)


def test_reference_arm_prints_one_json_line():
    r = _run()
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    sys.path.insert(0, ROOT)
    import bench
    assert d["metric"] == bench.METRIC == "FWI gradient shots/s, batched adjoint vs plain, 1\u00d7GB300 at \u22641e-3 rel err; Gcell/s"
    assert d["unit"] == "shots/s" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] == 2 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("cfg2")


def test_reference_arm_runs_on_rank_zero_only():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
