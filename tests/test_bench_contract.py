"""bench.py's output contract, on the CPU: the reference arm (the oracle port
timed on the host cores) prints one JSON line with the agreed keys, other
ranks print nothing, and the workload presets describe the configurations
they stand for."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def run_reference(extra_env=None, *args):
    env = dict(os.environ, **(extra_env or {}))
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "1", "--cpu-rays", "2000", "--points", "20000", "--views", "2", *args]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = run_reference()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    with open(os.path.join(ROOT, "BASELINE.json")) as f:
        assert line["metric"] == json.load(f)["metric"]
    assert line["impl"] == "reference"
    assert line["unit"] == "Mrays/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 1
    assert line["config"]["points"] == 20000 and line["config"]["views"] == 2
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_are_silent():
    r = run_reference({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


class _Args:
    def __init__(self, workload, points=None, views=None, resolution=None):
        self.workload, self.points, self.views, self.resolution = workload, points, views, resolution


def test_workload_presets():
    c2 = bench.workload_spec(_Args("c2"))
    assert (c2["points"], c2["boxes"], c2["density"], c2["views"]) == (20_000_000, 40, 1.0, 256)
    assert c2["res"] == [(640, 480), (1068, 690), (1920, 1080)]
    c4 = bench.workload_spec(_Args("c4"))
    assert (c4["points"], c4["boxes"], c4["density"], c4["views"], c4["res"]) == (100_000_000, 12, 100.0, 1024, None)
    assert "per-surface density log-uniform over 100x" in bench.workload_name(_Args("c4"), 100_000_000, 1024)
    small = bench.workload_spec(_Args("c2", points=1000, views=3, resolution="64x48"))
    assert (small["points"], small["views"], small["res"]) == (1000, 3, [(64, 48)])


@pytest.mark.parametrize("flag", ["--workload", "--impl"])
def test_argument_choices_are_closed(flag):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), flag, "bogus"], capture_output=True,
                       text=True, cwd=ROOT, timeout=120)
    assert r.returncode != 0 and "invalid choice" in r.stderr
