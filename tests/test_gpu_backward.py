"""Backward kernel: gradients of L = sum ||rgb - rgb*||^2 + sum |depth - depth*|
w.r.t. float32 colours, positions and radii through each pixel's stored hit.

Checks (the differentiable model is the first hit's colour and the analytic
entry distance into the hit sphere, hit held fixed):
  * FP64 central differences on 2000 random non-silhouette pixels (step
    1e-4 m for positions and radii, 1e-3 for colours), Richardson-
    extrapolated over h and h/2 so the check measures the kernel rather
    than the difference formula's truncation error: within 1e-4 relative;
  * a torch float64 autograd re-implementation of the same first-hit
    shading over every pixel: within 1e-4 relative (float32 atomics);
  * several views in one call equal the sum of per-view calls.
Targets are rendered from a copy with positions perturbed by N(0, 5 mm) and
colours by +-30, as in the differentiation workload.
"""
import numpy as np
import pytest
import torch

import oracle
from renderer_ray_marching_gb300 import Renderer, synthetic as syn, views_from_specs
from renderer_ray_marching_gb300.autograd import RenderFunction

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def setup():
    sc = syn.make_scene(300_000, n_boxes=12, seed=31)
    rng = np.random.default_rng(5)
    specs = syn.make_views(2, seed=12, boxes=sc.boxes, resolutions=[(320, 240)])
    views = views_from_specs(specs)
    r = Renderer()
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    radii, _ = r.compute_radii(0.1)
    rc = np.minimum(radii, np.float32(0.1))
    # targets from a perturbed copy
    xyz_t = (sc.xyz + rng.normal(0, 0.005, sc.xyz.shape)).astype(np.float32)
    rgb_t = np.clip(sc.rgb.astype(np.int32) + rng.integers(-30, 31, sc.rgb.shape), 0, 255).astype(np.uint8)
    rt = Renderer()
    rt.set_cloud(xyz_t, rgb_t)
    rt.build_index()
    rt.compute_radii(0.1)
    tgt = [rt.render(v, outputs=("rgbd", "hit")) for v in views]
    pred = [r.render(v, outputs=("rgbd", "hit")) for v in views]
    panes = r.view_pane(views)
    return sc, r, rc, views, pred, tgt, panes


def loss_grads(pred, tgt):
    """dL/drgb and dL/ddepth per pixel over pixels where both images hit."""
    rgbd = pred["rgbd"].reshape(-1, 4).astype(np.float64)
    trgbd = tgt["rgbd"].reshape(-1, 4).astype(np.float64)
    both = (pred["hit"].reshape(-1) >= 0) & (tgt["hit"].reshape(-1) >= 0)
    g_rgb = np.where(both[:, None], 2.0 * (rgbd[:, :3] - trgbd[:, :3]), 0.0).astype(np.float32)
    g_d = np.where(both, np.sign(rgbd[:, 3] - trgbd[:, 3]), 0.0).astype(np.float32)
    return g_rgb, g_d, both


def fd_check(sc, r, rc, v, pane, p, t, count, seed):
    """Backward of one view against FP64 central differences on `count`
    non-silhouette pixels with distinct hit points (Richardson over h, h/2
    for positions and radii); returns the worst relative error."""
    hit = p["hit"].reshape(-1).astype(np.int32)
    g_rgb_all, _, both = loss_grads(p, t)
    ov = oracle.make_view(v.cam2world, v.width, v.height, float(pane))
    col = sc.rgb.astype(np.float32) / np.float32(255.0)
    trgbd = t["rgbd"].reshape(-1, 4).astype(np.float64)
    rng = np.random.default_rng(seed)
    chosen, seen = [], set()
    for pix in rng.permutation(np.nonzero(both)[0]):
        h = int(hit[pix])
        if h in seen:
            continue
        o, d, _, _ = oracle.ray(ov, int(pix % v.width), int(pix // v.width))
        c = sc.xyz[h].astype(np.float64)
        rr = float(rc[h])
        tt, _, _, disc = oracle.sphere_depth(o.astype(np.float64), d.astype(np.float64), c, rr)
        a = float(np.dot(d.astype(np.float64), d.astype(np.float64)))
        # non-silhouette: the ray is well inside the sphere's disc and the
        # L1 term keeps its sign under the steps
        if disc <= 0.25 * a * rr * rr or abs(tt - trgbd[pix, 3]) < 1e-2:
            continue
        seen.add(h)
        chosen.append((int(pix), h, o.astype(np.float64), d.astype(np.float64)))
        if len(chosen) == count:
            break
    assert len(chosen) >= count // 2
    dl_rgb = np.zeros((v.pixels, 3), np.float32)
    dl_d = np.zeros(v.pixels, np.float32)
    for pix, h, o, d in chosen:
        tt, _, _, _ = oracle.sphere_depth(o, d, sc.xyz[h].astype(np.float64), float(rc[h]))
        dl_rgb[pix] = g_rgb_all[pix]
        dl_d[pix] = np.sign(tt - trgbd[pix, 3])
    n = sc.xyz.shape[0]
    gc, gx, gr = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32)
    r.backward([v], dl_rgb, dl_d, hit, gc, gx, gr)

    def pix_loss(pix, o, d, c, rr, colv):
        tt, _, _, _ = oracle.sphere_depth(o, d, c, rr)
        return float(np.sum((colv - trgbd[pix, :3]) ** 2) + abs(tt - trgbd[pix, 3]))

    def rich(f, h):
        d1 = (f(h) - f(-h)) / (2 * h)
        d2 = (f(h / 2) - f(-h / 2)) / h
        return (4 * d2 - d1) / 3

    worst = 0.0
    for pix, h, o, d in chosen:
        c0 = sc.xyz[h].astype(np.float64)
        r0 = float(rc[h])
        col0 = col[h].astype(np.float64)
        fd = np.zeros(7)
        for a in range(3):
            e = np.zeros(3)
            e[a] = 1.0
            fd[3 + a] = rich(lambda s: pix_loss(pix, o, d, c0 + s * e, r0, col0), 1e-4)
            fd[a] = (pix_loss(pix, o, d, c0, r0, col0 + 1e-3 * e) - pix_loss(pix, o, d, c0, r0, col0 - 1e-3 * e)) / 2e-3
        fd[6] = rich(lambda s: pix_loss(pix, o, d, c0, r0 + s, col0), 1e-4)
        got = np.concatenate([gc[h], gx[h], [gr[h]]]).astype(np.float64)
        scale = max(np.max(np.abs(fd[3:])), 1e-3)
        err_geo = np.max(np.abs(got[3:] - fd[3:])) / scale
        err_col = np.max(np.abs(got[:3] - fd[:3])) / max(np.max(np.abs(fd[:3])), 1e-3)
        worst = max(worst, err_geo, err_col)
    return worst, len(chosen)


def test_fd_fp64_non_silhouette(setup):
    sc, r, rc, views, pred, tgt, panes = setup
    worst, _ = fd_check(sc, r, rc, views[0], panes[0], pred[0], tgt[0], 2000, seed=0)
    assert worst <= TOL, worst


def test_fd_fp64_at_the_differentiation_workload_shape():
    """The differentiation workload's shape: a 1M-point cloud, 16 views at
    1067x690 (README intrinsics) of which 2 are checked, 1,000 non-silhouette
    pixels each (2,000 in all) against FP64 central differences."""
    sc = syn.make_scene(1_000_000, n_boxes=12, seed=4000)
    views = views_from_specs(syn.make_views(16, seed=4100, boxes=sc.boxes))
    assert all((v.width, v.height) == (1067, 690) for v in views)
    rng = np.random.default_rng(5)
    xyz_t = (sc.xyz + rng.normal(0, 0.005, sc.xyz.shape)).astype(np.float32)
    rgb_t = np.clip(sc.rgb.astype(np.int32) + rng.integers(-30, 31, sc.rgb.shape), 0, 255).astype(np.uint8)
    r = Renderer()
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    radii, _ = r.compute_radii(0.1)
    rc = np.minimum(radii, np.float32(0.1))
    rt = Renderer()
    rt.set_cloud(xyz_t, rgb_t)
    rt.build_index()
    rt.compute_radii(0.1)
    panes = r.view_pane(views)
    total = 0
    for i in (0, 1):
        p = r.render(views[i], outputs=("rgbd", "hit"))
        t = rt.render(views[i], outputs=("rgbd", "hit"))
        worst, k = fd_check(sc, r, rc, views[i], panes[i], p, t, 1000, seed=10 + i)
        assert worst <= TOL, (i, worst)
        total += k
    assert total >= 2000
    r.close()
    rt.close()


def test_autograd_reimplementation(setup):
    sc, r, rc, views, pred, tgt, panes = setup
    dev = torch.device("cuda:0")
    n = sc.xyz.shape[0]
    colours = torch.tensor(sc.rgb.astype(np.float32) / np.float32(255.0), device=dev, requires_grad=True)
    xyz = torch.tensor(sc.xyz, device=dev, requires_grad=True)
    radii = torch.tensor(rc, device=dev, requires_grad=True)
    rgb, depth, hit = RenderFunction.apply(r, views, colours, xyz, radii)
    trgbd = torch.cat([torch.tensor(t["rgbd"].reshape(-1, 4), device=dev) for t in tgt])
    thit = torch.cat([torch.tensor(t["hit"].reshape(-1), device=dev) for t in tgt])
    both = (hit >= 0) & (thit >= 0)
    loss = (((rgb - trgbd[:, :3]) ** 2).sum(1) * both).sum() + ((depth - trgbd[:, 3]).abs() * both).sum()
    loss.backward()
    # float64 re-implementation: colour gather + analytic entry distance, hit fixed
    sign = torch.where(both, torch.sign(depth.detach() - trgbd[:, 3]), torch.zeros_like(depth)).double()
    c64 = torch.tensor(sc.xyz, dtype=torch.float64, device=dev, requires_grad=True)
    r64 = torch.tensor(rc, dtype=torch.float64, device=dev, requires_grad=True)
    col64 = torch.tensor(sc.rgb.astype(np.float32) / np.float32(255.0), dtype=torch.float64, device=dev,
                         requires_grad=True)
    o_list, d_list = [], []
    for v, pane in zip(views, panes):
        ov = oracle.make_view(v.cam2world, v.width, v.height, float(pane))
        ys, xs = np.divmod(np.arange(v.pixels), v.width)
        od = [oracle.ray(ov, int(x), int(y)) for x, y in zip(xs, ys)]
        o_list.append(np.stack([a[0] for a in od]))
        d_list.append(np.stack([a[1] for a in od]))
    O = torch.tensor(np.concatenate(o_list), dtype=torch.float64, device=dev)
    D = torch.tensor(np.concatenate(d_list), dtype=torch.float64, device=dev)
    m = hit >= 0
    hm = hit[m].long()
    oc = c64[hm] - O[m]
    a = (D[m] * D[m]).sum(1)
    b = (D[m] * oc).sum(1)
    cc = (oc * oc).sum(1) - r64[hm] ** 2
    disc = b * b - a * cc
    inside = disc > 0
    t = torch.where(inside, (b - torch.sqrt(torch.clamp(disc, min=1e-300))) / a, b / a)
    rgb64 = col64[hm]
    loss64 = (((rgb64 - trgbd[m, :3].double()) ** 2).sum(1) * both[m]).sum() + (sign[m] * t).sum()
    loss64.backward()
    for got, ref in ((colours.grad, col64.grad), (xyz.grad, c64.grad), (radii.grad, r64.grad)):
        got = got.double()
        scale = ref.abs().max().clamp(min=1e-12)
        err = ((got - ref).abs().max() / scale).item()
        assert err <= TOL, err
    assert hit.shape[0] == sum(v.pixels for v in views) and n == xyz.grad.shape[0]


def test_multi_view_call_equals_sum_of_single_calls(setup):
    sc, r, rc, views, pred, tgt, panes = setup
    n = sc.xyz.shape[0]
    parts = [loss_grads(p, t) for p, t in zip(pred, tgt)]
    hits = [p["hit"].reshape(-1).astype(np.int32) for p in pred]
    one = [np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32)]
    r.backward(views, np.concatenate([q[0] for q in parts]), np.concatenate([q[1] for q in parts]),
               np.concatenate(hits), *one)
    two = [np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32)]
    for v, q, h in zip(views, parts, hits):
        r.backward([v], q[0], q[1], h, *two)
    for a, b in zip(one, two):
        # float32 atomics add in a different order: compare at 1e-4 of the largest entry
        assert np.max(np.abs(a - b)) <= TOL * max(np.max(np.abs(b)), 1e-6), (np.max(np.abs(a - b)), np.max(np.abs(b)))


def test_misses_and_bad_indices_give_zero_gradient(setup):
    sc, r, rc, views, pred, tgt, panes = setup
    n = sc.xyz.shape[0]
    v = views[0]
    hit = np.full(v.pixels, -1, np.int32)
    hit[:10] = n + 5  # outside the cloud: ignored
    g = [np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32)]
    r.backward([v], np.ones((v.pixels, 3), np.float32), np.ones(v.pixels, np.float32), hit, *g)
    assert all(np.all(x == 0) for x in g)
