"""Oracle self-checks on CPU: exact kNN against brute force, edge cases,
ray set-up, and the FP64 sphere-depth gradient against central differences."""
import math

import numpy as np
import pytest

import oracle
from tests.helpers import brute_knn


@pytest.mark.parametrize("n,k", [(1, 2), (5, 10), (12, 10), (400, 10), (400, 2), (257, 32)])
def test_knn_against_brute_force(n, k):
    rng = np.random.default_rng(n * 31 + k)
    xyz = rng.normal(size=(n, 3)).astype(np.float32)
    if n > 20:
        xyz[5:9] = xyz[2]          # duplicates: ties broken by lower index
        xyz[15, 0] = xyz[14, 0]    # shared coordinates
    q = np.concatenate([xyz[: min(n, 40)], rng.normal(size=(60, 3)).astype(np.float32) * 3])
    ix = oracle.Index(xyz)
    oi, od = ix.knn(q, k)
    bi, bd = brute_knn(xyz, q, k)
    assert np.array_equal(oi, bi)
    assert np.array_equal(od.view(np.int32), bd.view(np.int32))


def test_empty_cloud():
    ix = oracle.Index(np.zeros((0, 3), np.float32))
    oi, od = ix.knn(np.zeros((3, 3), np.float32), 4)
    assert np.all(oi == -1) and np.all(np.isinf(od))
    s, i = ix.distance(np.zeros(0, np.float32), [0, 0, 0])
    assert math.isinf(s) and i == 0


def test_single_point_radius_is_inf_then_clamped():
    ix = oracle.Index(np.array([[1.0, 2.0, 3.0]], np.float32))
    r, nn = ix.radii(0.0)
    assert np.isinf(r[0]) and nn[0] == -1
    r, _ = ix.radii(0.05)
    assert r[0] == np.float32(0.05)


def test_ray_setup_matches_pinhole():
    # identity pose: camera at origin looking down -Z
    m = np.eye(4, dtype=np.float32).T.reshape(16)
    w, h, pane = 64, 48, 50.0
    v = oracle.make_view(m, w, h, pane)
    o, d, tn, tf = oracle.ray(v, w // 2, h // 2)
    assert np.allclose(o, 0)
    assert np.allclose(d, [0, 0, -1])
    assert np.isclose(tn, 0.1) and np.isclose(tf, 100.0)
    o, d, tn, tf = oracle.ray(v, 0, 0)
    ref = np.array([-32.0, -24.0, -50.0])
    assert np.allclose(d, ref / np.linalg.norm(ref), atol=1e-6)
    assert tn > 0.1 and tf > 100.0


def test_sphere_depth_gradient_fd():
    rng = np.random.default_rng(3)
    for _ in range(50):
        o = rng.normal(size=3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = rng.uniform(0.002, 0.02)
        c = o + d * rng.uniform(0.5, 3.0) + rng.normal(size=3) * r * 0.3
        t, gc, gr, disc = oracle.sphere_depth(o, d, c, r)
        if disc <= 0:
            continue
        h = 1e-7
        for a in range(3):
            cp, cm = c.copy(), c.copy()
            cp[a] += h
            cm[a] -= h
            fd = (oracle.sphere_depth(o, d, cp, r)[0] - oracle.sphere_depth(o, d, cm, r)[0]) / (2 * h)
            assert abs(fd - gc[a]) < 1e-5 * max(1.0, abs(gc[a]))
        fd = (oracle.sphere_depth(o, d, c, r + h)[0] - oracle.sphere_depth(o, d, c, r - h)[0]) / (2 * h)
        assert abs(fd - gr) < 1e-5 * max(1.0, abs(gr))


def test_march_against_brute_force_rays():
    """Whole rays traced with an independent brute-force 10-NN agree exactly
    with the oracle's kd-tree march (hit, depth bits, step count)."""
    from renderer_ray_marching_gb300 import synthetic as syn
    from tests.helpers import brute_march
    sc = syn.make_scene(20000, n_boxes=8, seed=21)
    ix = oracle.Index(sc.xyz)
    radii, _ = ix.radii(0.1)
    spec = syn.make_views(1, seed=3, boxes=sc.boxes, resolutions=[(64, 48)])[0]
    m, w, h, fov = syn.view_params(spec)
    pane = np.float32(np.float32(w) / (np.float32(2.0) * np.float32(math.tan(np.float32(0.5) * fov))))
    v = oracle.make_view(m, w, h, pane)
    pix = np.random.default_rng(0).choice(w * h, 48, replace=False).astype(np.int64)
    hit, depth, steps = ix.render(radii, v, pix)
    for k, p in enumerate(pix):
        o, d, tn, tf = oracle.ray(v, int(p % w), int(p // w))
        bh, bd, bs = brute_march(sc.xyz, radii, o, d, tn, tf)
        assert (hit[k], steps[k]) == (bh, bs), (k, p)
        assert np.float32(depth[k]).view(np.int32) == np.float32(bd).view(np.int32)
    assert (hit >= 0).mean() > 0.3


def test_march_with_duplicate_points_against_brute_force():
    """A cloud in which many points are exact copies (equal distances at
    every step): the oracle's march keeps (d2, index) order and the strict
    '<' of the step value exactly as the brute-force loop does."""
    from renderer_ray_marching_gb300 import synthetic as syn
    from tests.helpers import brute_march
    sc = syn.make_scene(12000, n_boxes=6, seed=22)
    xyz = sc.xyz.copy()
    rng = np.random.default_rng(8)
    dst = rng.choice(xyz.shape[0], xyz.shape[0] // 2, replace=False)
    xyz[dst] = xyz[rng.integers(0, xyz.shape[0], dst.shape[0])]
    ix = oracle.Index(xyz)
    radii, _ = ix.radii(0.1)
    assert (radii == 0).mean() > 0.3
    spec = syn.make_views(1, seed=4, boxes=sc.boxes, resolutions=[(48, 32)])[0]
    m, w, h, fov = syn.view_params(spec)
    pane = np.float32(np.float32(w) / (np.float32(2.0) * np.float32(math.tan(np.float32(0.5) * fov))))
    v = oracle.make_view(m, w, h, pane)
    pix = np.random.default_rng(1).choice(w * h, 40, replace=False).astype(np.int64)
    hit, depth, steps = ix.render(radii, v, pix)
    for k, p in enumerate(pix):
        o, d, tn, tf = oracle.ray(v, int(p % w), int(p // w))
        bh, bd, bs = brute_march(xyz, radii, o, d, tn, tf)
        assert (hit[k], steps[k]) == (bh, bs), (k, p)
        assert np.float32(depth[k]).view(np.int32) == np.float32(bd).view(np.int32)
    assert (hit >= 0).mean() > 0.3
