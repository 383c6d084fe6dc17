"""GPU parity at the benchmark scales, against the CPU oracle.

The 100k-point tests in test_gpu_parity.py check every code path on a
shallow tree.  These run the configurations the benchmark reports on, at
full cloud size, and compare a seeded sample of pixels of every view with
the oracle's march (the reference's loop of src/ray_marching.cu:202-292 with
an exact 10-NN per step):

- the 2M-point cloud with max_radius 0.05 and 64 views at 1067x690
  rendered one view per launch (the plain form);
- the 20M-point cloud with 40 boxes, rendered in the batched form over views
  of all three resolutions; its index is 11 levels deep, and its best-first
  walks move pending nodes to the shared-memory overflow stack (counted).

Hit indices, depth bits and the step counts of hits must be identical; a
ray that misses may stop earlier on the GPU (exit culling), never later.
"""
import numpy as np
import pytest

import oracle
from renderer_ray_marching_gb300 import Renderer, synthetic as syn, views_from_specs

pytestmark = pytest.mark.gpu


def compare_sample(ix, radii_clamped, r, views, frames, per_view, seed):
    panes = r.view_pane(views)
    rng = np.random.default_rng(seed)
    rays = 0
    for v, f, pane in zip(views, frames, panes):
        pix = np.sort(rng.choice(v.pixels, min(per_view, v.pixels), replace=False)).astype(np.int64)
        oh, od, os_ = ix.render(radii_clamped, oracle.make_view(v.cam2world, v.width, v.height, float(pane)), pix)
        gh = f["hit"].reshape(-1)[pix]
        gd = f["depth"].reshape(-1)[pix]
        gs = f["steps"].reshape(-1)[pix]
        assert np.array_equal(gh, oh), "hit index differs at %d of %d pixels" % ((gh != oh).sum(), pix.size)
        assert np.array_equal(gd.view(np.int32), od.view(np.int32)), "depth bits differ"
        hit = oh >= 0
        assert np.array_equal(gs[hit], os_[hit]), "step counts of hits differ"
        assert np.all(gs[~hit] <= os_[~hit])
        rays += pix.size
    return rays


def test_c1_plain_views_match_oracle():
    """2M points, max_radius 0.05, 64 views at 1067x690, one rm_render each;
    1,500 sampled pixels per view (96,000 rays) against the oracle."""
    sc = syn.make_scene(2_000_000, n_boxes=12, seed=1000)
    views = views_from_specs(syn.make_views(64, seed=1100, boxes=sc.boxes))
    assert all((v.width, v.height) == (1067, 690) for v in views)
    r = Renderer(leaf_size=16)
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    radii, nn = r.compute_radii(0.05)
    ix = oracle.Index(sc.xyz)
    orad, onn = ix.radii(0.0)
    assert np.array_equal(radii.view(np.int32), orad.view(np.int32))
    assert np.array_equal(nn, onn)
    rc = np.minimum(orad, np.float32(0.05))
    frames = [r.render(v, outputs=("hit", "depth", "steps")) for v in views]
    st = r.stats()
    assert st["search_errors"] == 0
    rays = compare_sample(ix, rc, r, views, frames, 1500, seed=7)
    assert rays == 64 * 1500
    hit_frac = np.mean([(f["hit"] >= 0).mean() for f in frames])
    assert hit_frac > 0.9
    r.close()


def test_20M_batched_mixed_views_match_oracle():
    """20M points, 40 boxes (the batched workload's cloud), 8 views of
    640x480, 1068x690 and 1920x1080 in one batched launch; 20,000 sampled
    pixels per view (160,000 rays) against the oracle."""
    torch = pytest.importorskip("torch")
    sc = syn.make_scene(20_000_000, n_boxes=40, seed=2000)
    views = views_from_specs(syn.make_views(8, seed=3000, boxes=sc.boxes,
                                            resolutions=[(640, 480), (1068, 690), (1920, 1080)]))
    assert len({(v.width, v.height) for v in views}) == 3
    r = Renderer(leaf_size=16)
    r.set_cloud(torch.from_numpy(sc.xyz).cuda(), torch.from_numpy(sc.rgb).cuda())
    r.build_index()
    radii, nn = r.compute_radii(0.1, device=True)
    radii_h = radii.cpu().numpy()
    frames = r.render_batch(views, outputs=("hit", "depth", "steps"), device=False)
    st = r.stats()
    assert st["search_errors"] == 0
    assert st["rays"] == sum(v.pixels for v in views)
    # the walk's overflow stack was in use during the compared launch
    assert st["queue_spills"] > 0, st
    ix = oracle.Index(sc.xyz)
    # radii: a seeded sample of points against the oracle's exact 2-NN
    q = np.random.default_rng(3).choice(sc.xyz.shape[0], 200_000, replace=False)
    oi, od = ix.knn(sc.xyz[q], 2)
    assert np.array_equal(radii_h[q].view(np.int32), np.sqrt(od[:, 1], dtype=np.float32).view(np.int32))
    assert np.array_equal(nn.cpu().numpy()[q], oi[:, 1])
    rc = np.minimum(radii_h, np.float32(0.1))
    rays = compare_sample(ix, rc, r, views, frames, 20_000, seed=8)
    assert rays == 8 * 20_000
    r.close()
