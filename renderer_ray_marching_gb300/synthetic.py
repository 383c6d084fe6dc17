"""Seeded synthetic indoor scenes and camera views.

The reference ships no sample data, so every workload here is generated:
an axis-aligned room (x in [0, 8], y in [0, 6], z in [0, 3] metres, z up)
made of floor, ceiling and four walls, plus boxes with sides U[0.3, 1.5] m
resting on the floor.  Points are sampled uniformly by surface area (or
with a per-surface density drawn log-uniformly over a 100x range) and
jittered by N(0, 3 mm).  Each surface has a base colour U{0..255}^3 and
every point adds uniform integer noise in [-20, 20], clamped to uint8.

Views follow the reference's JSON conventions (README.md:38-98,
main.cu:193-206): ``camera_pose`` is a row-major camera-to-world matrix in
the OpenGL convention (-Z forward, +Y up) and ``calibration_mat`` a
row-major intrinsic matrix whose principal point is half the image size.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import dataclasses
import math

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.atanf.restype = ctypes.c_float
_libm.atanf.argtypes = [ctypes.c_float]


def atanf(x: float) -> np.float32:
    """C's float atanf, as the reference's host code calls it (main.cu:206)."""
    return np.float32(_libm.atanf(ctypes.c_float(float(x))))

ROOM = np.array([8.0, 6.0, 3.0])


@dataclasses.dataclass
class Scene:
    xyz: np.ndarray      # (N, 3) float32
    rgb: np.ndarray      # (N, 3) uint8
    boxes: np.ndarray    # (B, 6) float64: min xyz, max xyz
    seed: int


@dataclasses.dataclass
class ViewSpec:
    camera_pose: np.ndarray      # (4, 4) float64 row-major camera-to-world
    calibration_mat: np.ndarray  # (4, 4) float64 row-major intrinsics


def _surfaces(boxes: np.ndarray):
    """Rectangles as (origin, edge_u, edge_v) in metres."""
    X, Y, Z = ROOM
    rects = [
        ((0, 0, 0), (X, 0, 0), (0, Y, 0)),   # floor
        ((0, 0, Z), (X, 0, 0), (0, Y, 0)),   # ceiling
        ((0, 0, 0), (X, 0, 0), (0, 0, Z)),   # wall y=0
        ((0, Y, 0), (X, 0, 0), (0, 0, Z)),   # wall y=Y
        ((0, 0, 0), (0, Y, 0), (0, 0, Z)),   # wall x=0
        ((X, 0, 0), (0, Y, 0), (0, 0, Z)),   # wall x=X
    ]
    for b in boxes:
        x0, y0, z0, x1, y1, z1 = b
        sx, sy, sz = x1 - x0, y1 - y0, z1 - z0
        rects += [
            ((x0, y0, z1), (sx, 0, 0), (0, sy, 0)),   # top
            ((x0, y0, z0), (sx, 0, 0), (0, 0, sz)),   # side y0
            ((x0, y1, z0), (sx, 0, 0), (0, 0, sz)),   # side y1
            ((x0, y0, z0), (0, sy, 0), (0, 0, sz)),   # side x0
            ((x1, y0, z0), (0, sy, 0), (0, 0, sz)),   # side x1
        ]
    return [tuple(np.asarray(v, np.float64) for v in r) for r in rects]


def make_boxes(rng: np.random.Generator, n_boxes: int) -> np.ndarray:
    boxes = np.zeros((n_boxes, 6))
    for i in range(n_boxes):
        s = rng.uniform(0.3, 1.5, size=3)
        s[2] = min(s[2], ROOM[2] - 0.2)
        lo = rng.uniform([0.0, 0.0], ROOM[:2] - s[:2])
        boxes[i] = [lo[0], lo[1], 0.0, lo[0] + s[0], lo[1] + s[1], s[2]]
    return boxes


def make_scene(n_points: int, n_boxes: int = 12, seed: int = 0, jitter: float = 0.003,
               density_range: float = 1.0, chunk: int = 1 << 22) -> Scene:
    """Sample ``n_points`` on the room and box surfaces.

    ``density_range`` > 1 draws each surface's relative density
    log-uniformly from [1, density_range] (100 for the large uneven cloud).
    """
    rng = np.random.default_rng(seed)
    boxes = make_boxes(rng, n_boxes)
    rects = _surfaces(boxes)
    area = np.array([np.linalg.norm(np.cross(u, v)) for _, u, v in rects])
    weight = area.copy()
    if density_range > 1.0:
        weight *= np.exp(rng.uniform(0.0, math.log(density_range), size=len(rects)))
    weight /= weight.sum()
    base = rng.integers(0, 256, size=(len(rects), 3))
    counts = rng.multinomial(n_points, weight)
    xyz = np.empty((n_points, 3), np.float32)
    rgb = np.empty((n_points, 3), np.uint8)
    pos = 0
    for si, (o, u, v) in enumerate(rects):
        c = int(counts[si])
        done = 0
        while done < c:
            m = min(chunk, c - done)
            a = rng.random((m, 1))
            b = rng.random((m, 1))
            p = o + a * u + b * v + rng.normal(0.0, jitter, size=(m, 3))
            xyz[pos:pos + m] = p.astype(np.float32)
            col = base[si] + rng.integers(-20, 21, size=(m, 3))
            rgb[pos:pos + m] = np.clip(col, 0, 255).astype(np.uint8)
            pos += m
            done += m
    perm = rng.permutation(n_points)
    return Scene(xyz=xyz[perm], rgb=rgb[perm], boxes=boxes, seed=seed)


def calibration(width: int, height: int, f: float) -> np.ndarray:
    """Row-major intrinsics with the principal point at the image centre."""
    return np.array([[f, 0.0, width / 2.0, 0.0],
                     [0.0, f, height / 2.0, 0.0],
                     [0.0, 0.0, 1.0, 0.0],
                     [0.0, 0.0, 0.0, 1.0]])


REF_CALIBRATION = np.array([[803.802316909057, 0.0, 533.5, 0.0],
                            [0.0, 803.802316909057, 345.0, 0.0],
                            [0.0, 0.0, 1.0, 0.0],
                            [0.0, 0.0, 0.0, 1.0]])


def look_pose(centre, yaw: float, pitch: float) -> np.ndarray:
    """Row-major camera-to-world pose, GL convention, world z up."""
    f = np.array([math.cos(pitch) * math.cos(yaw), math.cos(pitch) * math.sin(yaw), math.sin(pitch)])
    right = np.cross(f, [0.0, 0.0, 1.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, f)
    m = np.eye(4)
    m[:3, 0] = right
    m[:3, 1] = up
    m[:3, 2] = -f
    m[:3, 3] = centre
    return m


def make_views(n_views: int, seed: int = 1, boxes: np.ndarray | None = None,
               resolutions=None, ref_intrinsics: bool = True) -> list[ViewSpec]:
    """Camera centres uniform in the room shrunk by 0.5 m (rejecting those
    within 0.2 m of a box), yaw U[0, 2pi), pitch U[-20, 20] degrees.

    With ``resolutions`` (list of (W, H)) each view draws one uniformly and
    uses fx = fy = 0.75 W with the principal point at the centre; otherwise
    the README's intrinsics (fx = 803.802, cx = 533.5, cy = 345) are used.
    """
    rng = np.random.default_rng(seed)
    views = []
    while len(views) < n_views:
        c = rng.uniform([0.5, 0.5, 0.5], ROOM - 0.5)
        if boxes is not None and len(boxes):
            inside = np.all((c >= boxes[:, :3] - 0.2) & (c <= boxes[:, 3:] + 0.2), axis=1)
            if inside.any():
                continue
        yaw = rng.uniform(0.0, 2.0 * math.pi)
        pitch = math.radians(rng.uniform(-20.0, 20.0))
        pose = look_pose(c, yaw, pitch)
        if resolutions is not None:
            w, h = resolutions[rng.integers(0, len(resolutions))]
            K = calibration(w, h, 0.75 * w)
        else:
            K = REF_CALIBRATION.copy()
        views.append(ViewSpec(camera_pose=pose, calibration_mat=K))
    return views


def view_params(spec: ViewSpec):
    """The reference's per-view set-up (main.cu:193-206, utils.cu:137-149).

    Returns (cam2world column-major float32[16], width, height, fov) where
    width = (int)(2 * cx), height = (int)(2 * cy) and
    fov = 2 * atanf(width_f / (2 * fx)) in float32.
    """
    pose = np.asarray(spec.camera_pose, np.float64).astype(np.float32)
    K = np.asarray(spec.calibration_mat, np.float64).astype(np.float32)
    colmajor = np.ascontiguousarray(pose.T).reshape(16)
    w_f = np.float32(2.0) * K[0, 2]
    h_f = np.float32(2.0) * K[1, 2]
    fx = K[0, 0]
    fov = np.float32(2.0) * atanf(w_f / (np.float32(2.0) * fx))
    return colmajor, int(w_f), int(h_f), np.float32(fov)


def views_json(specs: list[ViewSpec], names: list[str] | None = None, split: str = "train") -> dict:
    names = names or ["renders/view_%04d_color.png" % i for i in range(len(specs))]
    body = {n: {"calibration_mat": s.calibration_mat.tolist(), "camera_pose": s.camera_pose.tolist()}
            for n, s in zip(names, specs)}
    out = {"train": {}, "val": {}}
    out[split] = body
    return out
