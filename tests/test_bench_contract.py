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
    assert line["metric"] == bench.METRIC  # the same metric as the GPU arm's line
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
    assert c2["max_radius"] == 0.1
    c1 = bench.workload_spec(_Args("c1"))
    assert (c1["points"], c1["boxes"], c1["views"], c1["res"], c1["max_radius"]) == (2_000_000, 12, 64, None, 0.05)
    assert c2["res"] == [(640, 480), (1068, 690), (1920, 1080)]
    c4 = bench.workload_spec(_Args("c4"))
    assert (c4["points"], c4["boxes"], c4["density"], c4["views"], c4["res"]) == (100_000_000, 12, 100.0, 1024, None)
    assert "per-surface density log-uniform over 100x" in bench.workload_name(_Args("c4"), 100_000_000, 1024)
    small = bench.workload_spec(_Args("c2", points=1000, views=3, resolution="64x48"))
    assert (small["points"], small["views"], small["res"]) == (1000, 3, [(64, 48)])


def test_oracle_comparison_counts_every_kind_of_disagreement():
    import numpy as np
    oh = np.array([5, -1, 7, 9], np.int32)
    od = np.array([1.5, 0.0, 2.0, 3.0], np.float32)
    os_ = np.array([10, 128, 12, 4], np.int32)
    same = bench.compare_with_oracle([(oh, od, os_)], [(oh, od, os_)])
    assert same == {"rays": 4, "hit_mismatch": 0, "depth_bit_mismatch": 0, "step_mismatch_on_hits": 0,
                    "miss_steps_above_oracle": 0}
    gd = od.copy()
    gd[2] = np.nextafter(gd[2], np.float32(3))
    gs = os_.copy()
    gs[0] += 1
    gs[1] = 20  # a culled miss stops earlier: not counted
    gh = oh.copy()
    gh[3] = 8
    c = bench.compare_with_oracle([(gh, gd, gs)], [(oh, od, os_)])
    assert (c["hit_mismatch"], c["depth_bit_mismatch"], c["step_mismatch_on_hits"], c["miss_steps_above_oracle"]) == (
        1, 1, 1, 0)
    gs[1] = 129
    assert bench.compare_with_oracle([(oh, od, gs)], [(oh, od, os_)])["miss_steps_above_oracle"] == 1


@pytest.mark.parametrize("flag", ["--workload", "--impl"])
def test_argument_choices_are_closed(flag):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), flag, "bogus"], capture_output=True,
                       text=True, cwd=ROOT, timeout=120)
    assert r.returncode != 0 and "invalid choice" in r.stderr
