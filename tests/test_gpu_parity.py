"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bit-exact for neighbour indices, squared distances, radii, hit indices and
depths (the kernels and the oracle evaluate the same float32 operation
sequence); colour equals the hit point's uint8 colour / 255.
"""
import numpy as np
import pytest

import oracle
from renderer_ray_marching_gb300 import Renderer, synthetic as syn, views_from_specs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene100k():
    sc = syn.make_scene(100_000, n_boxes=12, seed=0)
    ix = oracle.Index(sc.xyz)
    return sc, ix


def make_renderer(xyz, rgb=None, leaf=16, max_radius=0.1, search=1):
    r = Renderer(leaf_size=leaf)
    r.set_launch(search=search)
    r.set_cloud(xyz, rgb)
    r.build_index()
    radii, nn = r.compute_radii(max_radius)
    return r, radii, nn


def oracle_view(r: Renderer, v):
    pane = r.view_pane([v])[0]
    return oracle.make_view(v.cam2world, v.width, v.height, float(pane))


@pytest.mark.parametrize("n", [1, 5, 12, 1000, 30000])
@pytest.mark.parametrize("k", [1, 2, 10, 16, 32])
def test_knn_bit_exact(n, k):
    rng = np.random.default_rng(n + 7 * k)
    xyz = rng.normal(size=(n, 3)).astype(np.float32)
    if n >= 12:
        xyz[3:7] = xyz[1]  # duplicates
    q = np.concatenate([xyz[: min(n, 200)], rng.normal(size=(300, 3)).astype(np.float32) * 2,
                        rng.normal(size=(20, 3)).astype(np.float32) * 100])
    r = Renderer()
    r.set_cloud(xyz)
    r.build_index()
    gi, gd = r.knn(q, k)
    oi, od = oracle.Index(xyz).knn(q, k)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd.view(np.int32), od.view(np.int32))


def test_knn_empty_cloud_pads():
    r = Renderer()
    r.set_cloud(np.zeros((0, 3), np.float32))
    r.build_index()
    gi, gd = r.knn(np.zeros((4, 3), np.float32), 3)
    assert np.all(gi == -1) and np.all(np.isinf(gd))


@pytest.mark.parametrize("leaf,search", [(8, 1), (16, 1), (32, 1), (16, 0)])
def test_radii_bit_exact(scene100k, leaf, search):
    sc, ix = scene100k
    r, radii, nn = make_renderer(sc.xyz, sc.rgb, leaf=leaf, search=search)
    orad, onn = ix.radii(0.0)
    assert np.array_equal(radii.view(np.int32), orad.view(np.int32))
    assert np.array_equal(nn, onn)


def test_radii_golden_flann_fixture():
    import os
    g = os.path.join(os.path.dirname(__file__), "golden")
    knn = np.load(os.path.join(g, "knn_flann.npz"))
    gold = np.load(os.path.join(g, "radii_flann.npz"))
    r, radii, nn = make_renderer(knn["xyz"])
    assert np.array_equal(radii.view(np.int32), gold["radii"].view(np.int32))
    assert np.array_equal(nn, gold["nn"])


def test_radii_single_point_and_clamp():
    r, radii, nn = make_renderer(np.array([[1, 2, 3]], np.float32), max_radius=0.05)
    assert np.isinf(radii[0]) and nn[0] == -1


def test_render_plain_matches_oracle(scene100k):
    sc, ix = scene100k
    r, radii, _ = make_renderer(sc.xyz, sc.rgb)
    v = views_from_specs(syn.make_views(1, seed=1, boxes=sc.boxes))[0]
    assert (v.width, v.height) == (1067, 690)
    out = r.render(v, outputs=("rgbd", "hit", "depth", "steps"))
    pix = np.random.default_rng(0).choice(v.pixels, 20000, replace=False).astype(np.int64)
    oh, od, os_ = ix.render(np.minimum(radii, np.float32(0.1)), oracle_view(r, v), pix)
    gh = out["hit"].reshape(-1)[pix]
    gd = out["depth"].reshape(-1)[pix]
    gs = out["steps"].reshape(-1)[pix]
    assert np.array_equal(gh, oh)
    assert np.array_equal(gd.view(np.int32), od.view(np.int32))
    # the exit culling only ever shortens rays that miss
    assert np.array_equal(gs[oh >= 0], os_[oh >= 0])
    assert np.all(gs[oh < 0] <= os_[oh < 0])
    # colour = uint8 / 255 of the hit point, depth in .w; background zero
    rgbd = out["rgbd"].reshape(-1, 4)
    hits = out["hit"].reshape(-1)
    m = hits >= 0
    assert m.mean() > 0.5
    col = (sc.rgb[hits[m]].astype(np.float32) / np.float32(255.0)).astype(np.float32)
    assert np.array_equal(rgbd[m, :3], col)
    assert np.array_equal(rgbd[m, 3], out["depth"].reshape(-1)[m])
    assert np.all(rgbd[~m] == 0)
    # work bound: a packet never walks the whole tree (border tiles hold idle
    # lanes whose bound is +inf; they must not vote)
    st = r.stats()
    assert st["search_errors"] == 0
    assert st["packet_nodes"] / max(st["warp_steps"], 1) < 100, st


def test_render_batch_equals_plain(scene100k):
    sc, _ = scene100k
    r, radii, _ = make_renderer(sc.xyz, sc.rgb)
    specs = syn.make_views(6, seed=9, boxes=sc.boxes, resolutions=[(160, 120), (213, 138), (96, 54)])
    views = views_from_specs(specs)
    plain = [r.render(v, outputs=("rgbd", "hit", "depth", "steps")) for v in views]
    for launch in [(8, 4, 1, 4, 1), (8, 4, 2, 4, 0), (4, 8, 4, 2, 1), (16, 2, 2, 8, 1), (8, 4, 1, 6, 1)]:
        r.set_launch(*launch)
        batch = r.render_batch(views, outputs=("rgbd", "hit", "depth", "steps"), device=False)
        for p, b in zip(plain, batch):
            for key in ("hit", "steps"):
                assert np.array_equal(p[key], b[key]), (launch, key)
            assert np.array_equal(p["rgbd"].view(np.int32), b["rgbd"].view(np.int32)), launch
    # a second replay of the cached graph gives the same answer
    again = r.render_batch(views, outputs=("hit",), device=False)
    for p, b in zip(plain, again):
        assert np.array_equal(p["hit"], b["hit"])


def test_render_independent_of_leaf_size_and_search(scene100k):
    sc, _ = scene100k
    v = views_from_specs(syn.make_views(1, seed=4, boxes=sc.boxes, resolutions=[(200, 150)]))[0]
    outs = []
    for leaf, search, ctas in ((8, 1, 4), (16, 1, 8), (32, 1, 6), (8, 1, 7), (16, 0, 4)):
        r, _, _ = make_renderer(sc.xyz, sc.rgb, leaf=leaf, search=search)
        r.set_launch(search=search, ctas_per_sm=ctas)
        outs.append(r.render(v))
    for o in outs[1:]:
        assert np.array_equal(o["hit"], outs[0]["hit"])
        assert np.array_equal(o["depth"].view(np.int32), outs[0]["depth"].view(np.int32))


@pytest.mark.parametrize("n", [0, 1, 5, 11])
def test_render_tiny_clouds(n):
    rng = np.random.default_rng(n)
    xyz = (rng.random((n, 3)) * [8, 6, 3]).astype(np.float32)
    r = Renderer()
    r.set_cloud(xyz)
    r.build_index()
    radii, _ = r.compute_radii(0.5)
    v = views_from_specs(syn.make_views(1, seed=2, resolutions=[(48, 32)]))[0]
    out = r.render(v, outputs=("hit", "depth", "steps"))
    if n == 0:
        assert np.all(out["hit"] == -1)
        return
    ix = oracle.Index(xyz)
    oh, od, os_ = ix.render(np.minimum(radii, np.float32(0.5)), oracle_view(r, v))
    assert np.array_equal(out["hit"].reshape(-1), oh)
    assert np.array_equal(out["depth"].reshape(-1).view(np.int32), od.view(np.int32))
    gs = out["steps"].reshape(-1)
    assert np.array_equal(gs[oh >= 0], os_[oh >= 0]) and np.all(gs[oh < 0] <= os_[oh < 0])


def test_cached_radii_path_equals_computed(scene100k):
    sc, _ = scene100k
    r, radii, _ = make_renderer(sc.xyz, sc.rgb)
    v = views_from_specs(syn.make_views(1, seed=5, boxes=sc.boxes, resolutions=[(120, 90)]))[0]
    a = r.render(v)
    r2 = Renderer()
    r2.set_cloud(sc.xyz, sc.rgb)
    r2.set_radii(radii, 0.1)       # radii before the index (main.cu:122-149 order)
    r2.build_index()
    b = r2.render(v)
    r3 = Renderer()
    r3.set_cloud(sc.xyz, sc.rgb)
    r3.build_index()
    r3.set_radii(radii, 0.1)       # radii after the index
    c = r3.render(v)
    for o in (b, c):
        assert np.array_equal(a["hit"], o["hit"])
        assert np.array_equal(a["depth"].view(np.int32), o["depth"].view(np.int32))


def test_errors_are_status_codes_not_exits():
    from renderer_ray_marching_gb300._abi import RmError
    r = Renderer()
    v = views_from_specs(syn.make_views(1, seed=2, resolutions=[(8, 8)]))[0]
    with pytest.raises(RmError, match="RM_ERR_STATE"):
        r.render(v)
    r.set_cloud(np.zeros((10, 3), np.float32))
    with pytest.raises(RmError, match="RM_ERR_INVALID"):
        r.set_radii(np.zeros(9, np.float32))
    with pytest.raises(RmError, match="RM_ERR_INVALID"):
        r.set_cloud(np.array([[0, np.nan, 0]], np.float32)) or r.build_index()
    with pytest.raises(RmError, match="RM_ERR_INVALID"):
        r.set_launch(8, 8, 1, 4)


def test_pinned_host_frames_equal_device_frames(scene100k):
    """Host frames in pinned memory are written by the kernel directly; the
    result must equal device frames (and pageable host frames) bit for bit."""
    torch = pytest.importorskip("torch")
    import ctypes
    from renderer_ray_marching_gb300 import _abi
    sc, _ = scene100k
    r, _, _ = make_renderer(sc.xyz, sc.rgb)
    views = views_from_specs(syn.make_views(3, seed=17, boxes=sc.boxes, resolutions=[(160, 120), (97, 61)]))
    cviews = (_abi.RmView * len(views))(*[v.to_c() for v in views])
    fields = (("rgbd", 4, torch.float32), ("hit", 1, torch.int32), ("depth", 1, torch.float32),
              ("steps", 1, torch.int32))

    def frames(kind):
        arr = (_abi.RmFrame * len(views))()
        keep = []
        for i, v in enumerate(views):
            b = {}
            for name, ch, dt in fields:
                shape = (v.height, v.width, ch) if ch > 1 else (v.height, v.width)
                if kind == "device":
                    t = torch.full(shape, -3, dtype=dt, device="cuda:0")
                else:
                    t = torch.full(shape, -3, dtype=dt)
                    if kind == "pinned":
                        t = t.pin_memory()
                setattr(arr[i], name, t.data_ptr())
                b[name] = t
            keep.append(b)
        return arr, keep

    def host(keep):
        return [{k: t.cpu().numpy().copy() for k, t in b.items()} for b in keep]

    out = {}
    for kind in ("device", "pinned", "pageable"):
        arr, keep = frames(kind)
        loc = _abi.RM_DEVICE if kind == "device" else _abi.RM_HOST
        _abi.check(r._lib, r._h, r._lib.rm_render_batch(r._h, cviews, len(views), arr, loc))
        r.synchronize()
        out["batch_" + kind] = host(keep)
        arr, keep = frames(kind)
        for i in range(len(views)):
            _abi.check(r._lib, r._h, r._lib.rm_render(r._h, ctypes.byref(cviews[i]), ctypes.byref(arr[i]), loc))
        r.synchronize()
        out["plain_" + kind] = host(keep)
    ref = out["batch_device"]
    for key, frames_ in out.items():
        for a, b in zip(ref, frames_):
            for name in ("hit", "steps"):
                assert np.array_equal(a[name], b[name]), (key, name)
            for name in ("rgbd", "depth"):
                assert np.array_equal(a[name].view(np.int32), b[name].view(np.int32)), (key, name)
    r.close()


@pytest.mark.parametrize("search", [1, 0])
def test_render_with_duplicate_points_matches_oracle(search):
    """40% of the points are exact copies of others, so equal distances are
    everywhere: the neighbour set's ordered path (ties by cloud index,
    duplicates skipped) and the tie pass of its re-sort both run."""
    sc = syn.make_scene(60_000, n_boxes=8, seed=11)
    xyz = sc.xyz.copy()
    rng = np.random.default_rng(5)
    dst = rng.choice(xyz.shape[0], xyz.shape[0] * 2 // 5, replace=False)
    xyz[dst] = xyz[rng.integers(0, xyz.shape[0], dst.shape[0])]
    r, radii, nn = make_renderer(xyz, sc.rgb, search=search)
    ix = oracle.Index(xyz)
    orad, onn = ix.radii(0.0)
    assert np.array_equal(radii.view(np.int32), orad.view(np.int32))
    assert np.array_equal(nn, onn)
    assert (radii == 0).mean() > 0.2  # duplicates have a zero radius
    rc = np.minimum(radii, np.float32(0.1))
    views = views_from_specs(syn.make_views(2, seed=6, boxes=sc.boxes, resolutions=[(160, 120), (96, 64)]))
    batch = r.render_batch(views, outputs=("hit", "depth", "steps"), device=False)
    for v, b in zip(views, batch):
        plain = r.render(v, outputs=("hit", "depth", "steps"))
        oh, od, os_ = ix.render(rc, oracle_view(r, v))
        for out in (plain, b):
            gh, gd, gs = out["hit"].reshape(-1), out["depth"].reshape(-1), out["steps"].reshape(-1)
            assert np.array_equal(gh, oh)
            assert np.array_equal(gd.view(np.int32), od.view(np.int32))
            assert np.array_equal(gs[oh >= 0], os_[oh >= 0]) and np.all(gs[oh < 0] <= os_[oh < 0])
        assert (oh >= 0).mean() > 0.5
    assert r.stats()["search_errors"] == 0
    r.close()


@pytest.mark.parametrize("offset", [1e4, -3.7e3])
def test_exit_culling_on_a_cloud_far_from_the_origin(offset):
    """The exit clip (every ray stops where it leaves the box of all centres
    grown by max radius + MIN_DIST + slack) must not change any result when
    float spacing is coarse: the room and the cameras moved 10^4 m (spacing
    about 1 mm, the size of MIN_DIST) or -3.7 km from the origin.  Every
    pixel of the view is compared with the oracle, which has no clip."""
    import dataclasses
    sc = syn.make_scene(100_000, n_boxes=12, seed=21)
    xyz = (sc.xyz.astype(np.float64) + offset).astype(np.float32)
    specs = syn.make_views(3, seed=22, boxes=sc.boxes, resolutions=[(200, 150)])
    moved = []
    for s in specs:
        pose = np.array(s.camera_pose, np.float64)
        pose[:3, 3] += offset
        moved.append(dataclasses.replace(s, camera_pose=pose))
    views = views_from_specs(moved)
    r, radii, _ = make_renderer(xyz, sc.rgb)
    ix = oracle.Index(xyz)
    orad, _ = ix.radii(0.0)
    assert np.array_equal(radii.view(np.int32), orad.view(np.int32))
    rc = np.minimum(radii, np.float32(0.1))
    for v, b in zip(views, r.render_batch(views, outputs=("hit", "depth", "steps"), device=False)):
        oh, od, os_ = ix.render(rc, oracle_view(r, v))
        gh, gd, gs = b["hit"].reshape(-1), b["depth"].reshape(-1), b["steps"].reshape(-1)
        assert np.array_equal(gh, oh)
        assert np.array_equal(gd.view(np.int32), od.view(np.int32))
        assert np.array_equal(gs[oh >= 0], os_[oh >= 0])
        assert np.all(gs[oh < 0] <= os_[oh < 0])
        assert (oh >= 0).mean() > 0.5
    assert r.stats()["search_errors"] == 0
    r.close()
