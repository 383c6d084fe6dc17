"""Host file formats of the reference's process boundary, on CPU."""
import os

import numpy as np
import pytest

from renderer_ray_marching_gb300 import fileio
from tests.pngread import read_png


def test_ply_binary_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    xyz = rng.normal(size=(1000, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (1000, 3)).astype(np.uint8)
    p = str(tmp_path / "c.ply")
    fileio.save_ply(p, xyz, rgb)
    x2, c2 = fileio.load_ply(p)
    assert np.array_equal(x2, xyz) and np.array_equal(c2, rgb)


def test_ply_ascii_and_double_coordinates(tmp_path):
    p = tmp_path / "a.ply"
    p.write_text("ply\nformat ascii 1.0\ncomment x\nelement vertex 2\nproperty double x\nproperty double y\n"
                 "property double z\nproperty float nx\nproperty uchar red\nproperty uchar green\n"
                 "property uchar blue\nelement face 0\nproperty list uchar int vertex_indices\nend_header\n"
                 "0.1 0.2 0.30000000000000004 1 10 20 30\n1e-3 -2 3.5 0 255 0 7\n")
    x, c = fileio.load_ply(str(p))
    # happly reads doubles; glm::vec4 narrows to float
    assert np.array_equal(x, np.array([[0.1, 0.2, 0.30000000000000004], [1e-3, -2, 3.5]]).astype(np.float32))
    assert np.array_equal(c, [[10, 20, 30], [255, 0, 7]])


def test_ply_big_endian_and_missing_colour(tmp_path):
    xyz = np.array([[1.5, -2.25, 3.0], [4, 5, 6]], ">f4")
    p = tmp_path / "b.ply"
    p.write_bytes(b"ply\nformat binary_big_endian 1.0\nelement vertex 2\nproperty float x\nproperty float y\n"
                  b"property float z\nend_header\n" + xyz.tobytes())
    x, c = fileio.load_ply(str(p))
    assert np.array_equal(x, xyz.astype(np.float32)) and np.all(c == 255)


def test_ply_errors(tmp_path):
    p = tmp_path / "bad.ply"
    p.write_text("not a ply\n")
    with pytest.raises(RuntimeError, match="bad magic"):
        fileio.load_ply(str(p))
    p.write_bytes(b"ply\nformat binary_little_endian 1.0\nelement vertex 5\nproperty float x\nproperty float y\n"
                  b"property float z\nend_header\n" + b"\0" * 20)
    with pytest.raises(RuntimeError, match="truncated"):
        fileio.load_ply(str(p))


def test_radii_archive_round_trip_exact(tmp_path):
    r = np.random.default_rng(1).random(5000).astype(np.float32) * np.float32(0.1)
    r[3] = np.inf
    r[4] = 0.0
    p = str(tmp_path / "x.ply.kdtree.radii")
    fileio.write_radii(p, r)
    assert open(p).read().startswith("22 serialization::archive 17 0 0 5000 0 ")
    back = fileio.read_radii(p)
    assert np.array_equal(back.view(np.int32), r.view(np.int32))


@pytest.mark.parametrize("body", ["0 0 3 0 1.5 2.5 3.5", "3 0 1.5 2.5 3.5", "3 1.5 2.5 3.5", "0 0 3 1.5 2.5 3.5"])
def test_radii_archive_layouts(tmp_path, body):
    p = tmp_path / "r.radii"
    p.write_text("22 serialization::archive 17 " + body + "\n")
    assert np.array_equal(fileio.read_radii(str(p)), np.array([1.5, 2.5, 3.5], np.float32))


def test_radii_archive_errors(tmp_path):
    p = tmp_path / "r.radii"
    p.write_text("22 serialization::archive 17 0 0 9 0 1 2 3\n")
    with pytest.raises(RuntimeError, match="count"):
        fileio.read_radii(str(p))
    p.write_text("hello")
    with pytest.raises(RuntimeError, match="Boost"):
        fileio.read_radii(str(p))


def test_frame_encoders(tmp_path):
    h, w = 5, 7
    rng = np.random.default_rng(2)
    rgbd = rng.random((h, w, 4)).astype(np.float32)
    rgbd[..., 3] *= 150.0
    rgbd[0, 0] = 0.0                     # background
    rgbd[1, 1, 3] = 1.0 + 5e-6           # "empty space" depth rule
    rgbd[2, 2, 3] = 120.0                # clamped to 255
    c, d = str(tmp_path / "v_color.png"), str(tmp_path / "v_depth.png")
    fileio.write_frame(c, d, rgbd)
    col = read_png(c)
    flipped = rgbd[::-1]
    assert np.array_equal(col[..., :3], (flipped[..., :3] * np.float32(255.0)).astype(np.uint8))
    assert np.all(col[..., 3] == 255)
    dep = read_png(d)
    v = flipped[..., 3]
    ref = np.clip(np.float32(2.55) * v, 0, 255).astype(np.uint8)
    ref[np.abs(v - np.float32(1.0)) < np.float32(1e-5)] = 0
    assert np.array_equal(dep, ref)
    npy = np.load(d + ".npy")
    assert npy.dtype == np.float32 and npy.shape == (h, w) and np.array_equal(npy, v)


def test_large_frame_pngs_deflated_in_slices(tmp_path):
    """A frame of 1920x1080 is deflated in row slices on several threads (one
    zlib stream: slices end on a sync flush, Adler-32 sums combined); the
    standard decoder (which checks the stream's checksum) gives the same
    pixels, and the stream holds more than one deflate segment."""
    h, w = 1080, 1920
    rng = np.random.default_rng(5)
    rgbd = np.zeros((h, w, 4), np.float32)
    rgbd[..., :3] = rng.integers(0, 4, size=(h, w, 3)).astype(np.float32) / np.float32(3.0)  # compressible
    rgbd[..., 3] = rng.random((h, w)).astype(np.float32) * np.float32(90.0)
    rgbd[: h // 3, :, 3] = 0.0
    c, d = str(tmp_path / "big_color.png"), str(tmp_path / "big_depth.png")
    fileio.write_frame(c, d, rgbd)
    col = read_png(c)
    flipped = rgbd[::-1]
    assert np.array_equal(col[..., :3], (flipped[..., :3] * np.float32(255.0)).astype(np.uint8))
    assert np.all(col[..., 3] == 255)
    dep = read_png(d)
    v = flipped[..., 3]
    ref = np.clip(np.float32(2.55) * v, 0, 255).astype(np.uint8)
    ref[np.abs(v - np.float32(1.0)) < np.float32(1e-5)] = 0
    assert np.array_equal(dep, ref)
    if (os.cpu_count() or 1) > 1:
        # a sync flush leaves an empty stored block (00 00 ff ff) between slices
        data = open(c, "rb").read()
        assert b"\x00\x00\xff\xff" in data


def test_json_rows_become_columns():
    m = fileio.json_mat4("[[1,2,3,4],[5,6,7,8],[9,10,11,12],[13,14,15,16]]")
    assert np.array_equal(m.reshape(4, 4).T, np.arange(1, 17, dtype=np.float32).reshape(4, 4))
    with pytest.raises(RuntimeError):
        fileio.json_mat4("[[1,2],[3]]")


def test_writers_report_unwritable_paths(tmp_path):
    """A writer that cannot create its file raises instead of passing silently."""
    missing = tmp_path / "no" / "such" / "dir"
    with pytest.raises(RuntimeError, match="cannot write"):
        fileio.write_radii(str(missing / "a.radii"), np.ones(4, np.float32))
    rgbd = np.zeros((3, 5, 4), np.float32)
    with pytest.raises(RuntimeError, match="cannot write"):
        fileio.write_frame(str(missing / "c.png"), str(missing / "c_depth.png"), rgbd)


def test_radii_archive_parallel_paths_are_exact(tmp_path):
    """Above about 10^6 values the archive is written and parsed in parallel
    slices: the bytes must equal one ' %.9e' per value in order, and any of
    the accepted layouts must parse back exactly."""
    rng = np.random.default_rng(3)
    r = (rng.random(1_200_000) * 0.1).astype(np.float32)
    r[::997] = 0.0
    p = tmp_path / "big.radii"
    fileio.write_radii(str(p), r)
    text = "22 serialization::archive 17 0 0 %d 0" % r.size + "".join(" %.9e" % v for v in r.tolist()) + "\n"
    assert p.read_text() == text
    assert np.array_equal(fileio.read_radii(str(p)).view(np.int32), r.view(np.int32))
    # layout without class information or item version, values split over lines
    body = "22 serialization::archive 17 %d" % r.size + "".join(
        ("\n" if i % 1000 == 0 else " ") + ("%.9e" % v) for i, v in enumerate(r.tolist()))
    q = tmp_path / "plain.radii"
    q.write_text(body)
    assert np.array_equal(fileio.read_radii(str(q)).view(np.int32), r.view(np.int32))
    q.write_text(body.replace(" 1.", " x.", 1))
    with pytest.raises(RuntimeError, match="bad value"):
        fileio.read_radii(str(q))


@pytest.mark.parametrize("order", ["<", ">"])
def test_ply_parallel_decode_large(tmp_path, order):
    """Above about 10^6 vertices the binary records are decoded in parallel
    slices; both byte orders and mixed property types must come out exact."""
    n = 1_200_000
    rng = np.random.default_rng(7)
    dt = np.dtype([("x", order + "f8"), ("y", order + "f4"), ("z", order + "f4"), ("nx", order + "f4"),
                   ("red", "u1"), ("green", "u1"), ("blue", "u1")])
    rec = np.zeros(n, dt)
    for k in ("x", "y", "z", "nx"):
        rec[k] = rng.normal(size=n)
    for k in ("red", "green", "blue"):
        rec[k] = rng.integers(0, 256, n)
    fmt = "binary_little_endian" if order == "<" else "binary_big_endian"
    header = ("ply\nformat %s 1.0\nelement vertex %d\nproperty double x\nproperty float y\nproperty float z\n"
              "property float nx\nproperty uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n" % (fmt, n))
    p = tmp_path / "big.ply"
    p.write_bytes(header.encode() + rec.tobytes())
    xyz, rgb = fileio.load_ply(str(p))
    want = np.stack([rec["x"].astype(np.float32), rec["y"].astype(np.float32), rec["z"].astype(np.float32)], 1)
    assert np.array_equal(xyz, want)
    assert np.array_equal(rgb, np.stack([rec["red"], rec["green"], rec["blue"]], 1))
