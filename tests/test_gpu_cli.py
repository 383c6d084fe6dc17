"""marcher.bin end to end: the reference's CLI, files and stdout protocol
(main.cu:56-275) over the CUDA library."""
import fcntl
import json
import os
import subprocess

import numpy as np
import pytest

from renderer_ray_marching_gb300 import Renderer, build, fileio, synthetic as syn, views_from_specs
from tests.pngread import read_png

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    sc = syn.make_scene(50_000, n_boxes=8, seed=77)
    ply = str(d / "scan.ply")
    fileio.save_ply(ply, sc.xyz, sc.rgb)
    specs = syn.make_views(3, seed=8, boxes=sc.boxes, resolutions=[(64, 48)])
    m = {"train": {"renders/a_color.png": {"calibration_mat": specs[0].calibration_mat.tolist(),
                                           "camera_pose": specs[0].camera_pose.tolist()},
                   "renders/b_color.png": {"calibration_mat": specs[1].calibration_mat.tolist(),
                                           "camera_pose": specs[1].camera_pose.tolist(),
                                           "source_scan_ply_path": ply}},
         "val": {"renders/c_color.png": {"calibration_mat": specs[2].calibration_mat.tolist(),
                                         "camera_pose": specs[2].camera_pose.tolist()},
                 "renders/z_color.png": {"calibration_mat": specs[2].calibration_mat.tolist(),
                                         "camera_pose": specs[2].camera_pose.tolist(),
                                         "source_scan_ply_path": str(d / "other.ply")}}}
    (d / "other.ply").write_text("")
    mj = str(d / "views.json")
    json.dump(m, open(mj, "w"))
    return d, sc, ply, mj, specs


def run(args):
    build.build()
    r = subprocess.run([build.CLI] + args, capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout, r.stderr


def test_cli_end_to_end(workdir):
    d, sc, ply, mj, specs = workdir
    out = str(d / "out")
    rc, so, se = run(["-f", ply, "-m", mj, "-o", out, "-d"])
    assert rc == 0, se
    lines = so.splitlines()
    assert lines[0] == "Number of points: 50000"
    assert lines[1] == "Precomputing radii..."
    assert lines[2] == "Matrices loaded."
    a = os.path.abspath(os.path.join(out, "renders", "a_color.png"))
    assert '"%s": LOCKING' % a in lines
    assert any(l.startswith('"%s": ' % os.path.realpath(a)) and l.endswith(" s") for l in lines)
    assert any(l.startswith("Skipping ") and "rerun with proper ply." in l for l in lines)
    assert not os.path.exists(os.path.join(out, "renders", "z_color.png"))
    # the radii cache equals the library's radii
    cache = fileio.read_radii(ply + ".kdtree.radii")
    r = Renderer()
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    radii, _ = r.compute_radii(0.1)
    assert np.array_equal(cache.view(np.int32), radii.view(np.int32))
    # images equal the library render encoded the reference's way
    for name, spec in (("a", specs[0]), ("b", specs[1]), ("c", specs[2])):
        v = views_from_specs([spec])[0]
        ref = r.render(v, outputs=("rgbd",))["rgbd"]
        col = read_png(os.path.join(out, "renders", name + "_color.png"))
        assert np.array_equal(col[..., :3], (ref[::-1, :, :3] * np.float32(255.0)).astype(np.uint8))
        dep = np.load(os.path.join(out, "renders", name + "_depth.png.npy"))
        assert np.array_equal(dep, ref[::-1, :, 3])
        assert read_png(os.path.join(out, "renders", name + "_depth.png")).shape == (48, 64)
        assert not os.path.exists(os.path.join(out, "renders", "." + name + "_color.png.lock"))

    # second run: cached radii, outputs skipped
    rc, so, se = run(["-f", ply, "-m", mj, "-o", out, "-d"])
    assert rc == 0, se
    assert "Using precomputed radii..." in so
    assert so.count("ALREADY EXISTS") == 3

    # batched form with -i rewrites identical images
    before = open(os.path.join(out, "renders", "b_color.png"), "rb").read()
    rc, so, se = run(["-f", ply, "-m", mj, "-o", out, "-d", "-i", "--batch"])
    assert rc == 0, se
    assert open(os.path.join(out, "renders", "b_color.png"), "rb").read() == before


def test_cli_respects_foreign_lock(workdir):
    d, sc, ply, mj, specs = workdir
    out = str(d / "out_lock")
    os.makedirs(os.path.join(out, "renders"))
    lp = os.path.join(out, "renders", ".a_color.png.lock")
    fd = os.open(lp, os.O_RDWR | os.O_CREAT)
    fcntl.lockf(fd, fcntl.LOCK_EX | fcntl.LOCK_NB)
    try:
        rc, so, se = run(["-f", ply, "-m", mj, "-o", out, "-d"])
    finally:
        fcntl.lockf(fd, fcntl.LOCK_UN)
        os.close(fd)
    assert rc == 0, se
    assert "ALREADY LOCKED" in so
    assert not os.path.exists(os.path.join(out, "renders", "a_color.png"))
    assert os.path.exists(os.path.join(out, "renders", "b_color.png"))


def test_cli_radii_count_mismatch_fails_cleanly(workdir):
    d, sc, ply, mj, specs = workdir
    bad = str(d / "small.ply")
    fileio.save_ply(bad, sc.xyz[:100], sc.rgb[:100])
    fileio.write_radii(bad + ".kdtree.radii", np.ones(99, np.float32))
    rc, so, se = run(["-f", bad, "-m", mj, "-o", str(d / "o3"), "-d"])
    assert rc != 0 and "does not contain the same number of points" in se


def test_cli_batch_write_error_keeps_other_views(workdir):
    """--batch: a view whose files cannot be written makes the run fail, but
    every other view is still reported and unlocked (only the failed view
    keeps its .lock file, as a run of the reference stopping there would)."""
    d, sc, ply, mj, specs = workdir
    out = str(d / "out_err")
    os.makedirs(os.path.join(out, "renders", "b_depth.png.npy"))  # the .npy path is a directory
    rc, so, se = run(["-f", ply, "-m", mj, "-o", out, "-d", "--batch"])
    assert rc != 0
    for name in ("a", "c"):
        p = os.path.realpath(os.path.join(out, "renders", name + "_color.png"))
        assert any(l.startswith('"%s": ' % p) and l.endswith(" s") for l in so.splitlines()), so
        assert os.path.exists(os.path.join(out, "renders", name + "_depth.png"))
        assert not os.path.exists(os.path.join(out, "renders", "." + name + "_color.png.lock"))
    assert os.path.exists(os.path.join(out, "renders", ".b_color.png.lock"))

