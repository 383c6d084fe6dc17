"""rm_render_batch_noalloc (the allocation-free batched form) against
rm_render_batch, through the C ABI.

The allocation-free entry point keeps its scratch in one static device
array that every call reuses, so the check runs two calls in a row with
different view sets and compares each with rm_render_batch on the same
context.  Results must be identical (hit indices, step counts and the bits
of colour and depth), the tolerance of the other marcher parity tests.
"""

import numpy as np
import pytest

from renderer_ray_marching_gb300 import Renderer, _abi, synthetic as syn, views_from_specs

pytestmark = pytest.mark.gpu

FIELDS = (("rgbd", 4, "f"), ("hit", 1, "i"), ("depth", 1, "f"), ("steps", 1, "i"))


def device_frames(torch, views, fill):
    frames = (_abi.RmFrame * len(views))()
    bufs = []
    for i, v in enumerate(views):
        b = {}
        for name, ch, kind in FIELDS:
            shape = (v.height, v.width, ch) if ch > 1 else (v.height, v.width)
            t = torch.full(shape, fill, dtype=torch.float32 if kind == "f" else torch.int32, device="cuda:0")
            setattr(frames[i], name, t.data_ptr())
            b[name] = t
        bufs.append(b)
    return frames, bufs


def host(bufs):
    return [{k: t.cpu().numpy() for k, t in b.items()} for b in bufs]


def test_noalloc_matches_batched_render_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    sc = syn.make_scene(60_000, n_boxes=8, seed=3)
    r = Renderer(leaf_size=16)
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    r.compute_radii(0.1)
    lib, h = r._lib, r._h
    view_sets = [
        views_from_specs(syn.make_views(6, seed=21, boxes=sc.boxes,
                                        resolutions=[(160, 120), (213, 138), (96, 54)])),
        views_from_specs(syn.make_views(3, seed=22, boxes=sc.boxes, resolutions=[(131, 77), (64, 200)])),
    ]
    for views in view_sets:
        cviews = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        ref_frames, ref_bufs = device_frames(torch, views, -5)
        _abi.check(lib, h, lib.rm_render_batch(h, cviews, len(views), ref_frames, _abi.RM_DEVICE))
        r.synchronize()
        # sentinel fill: every pixel must be written by the call itself
        na_frames, na_bufs = device_frames(torch, views, -7)
        torch.cuda.synchronize()
        _abi.check(lib, h, lib.rm_render_batch_noalloc(h, cviews, len(views), na_frames))
        for ref, got in zip(host(ref_bufs), host(na_bufs)):
            assert np.array_equal(ref["hit"], got["hit"])
            assert np.array_equal(ref["steps"], got["steps"])
            assert np.array_equal(ref["rgbd"].view(np.int32), got["rgbd"].view(np.int32))
            assert np.array_equal(ref["depth"].view(np.int32), got["depth"].view(np.int32))
            assert (got["hit"] >= 0).any()
        # its counters stay in the static scratch: the context's statistics
        # report zeros, not the previous rm_render_batch's figures
        st = r.stats()
        assert st["rays"] == 0 and st["steps"] == 0 and st["kernel_ms"] == 0.0
    r.close()


def test_noalloc_allocates_no_device_memory():
    """The device's free memory is the same before and after a call (after a
    first call on another view set, which loads the kernels), and a batch of
    exactly RM_NOALLOC_MAX_VIEWS views, which fills the static view table,
    still equals rm_render_batch."""
    torch = pytest.importorskip("torch")
    sc = syn.make_scene(30_000, n_boxes=6, seed=8)
    r = Renderer(leaf_size=16)
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    r.compute_radii(0.1)
    lib, h = r._lib, r._h
    small = views_from_specs(syn.make_views(4, seed=30, boxes=sc.boxes, resolutions=[(40, 24)]))
    full = views_from_specs(syn.make_views(_abi.RM_NOALLOC_MAX_VIEWS, seed=31, boxes=sc.boxes,
                                           resolutions=[(16, 8), (8, 12), (24, 4)]))
    c_small = (_abi.RmView * len(small))(*[v.to_c() for v in small])
    c_full = (_abi.RmView * len(full))(*[v.to_c() for v in full])
    f_small, b_small = device_frames(torch, small, -7)
    f_full, b_full = device_frames(torch, full, -7)
    ref_frames, ref_bufs = device_frames(torch, full, -5)
    torch.cuda.synchronize()
    _abi.check(lib, h, lib.rm_render_batch_noalloc(h, c_small, len(small), f_small))
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    _abi.check(lib, h, lib.rm_render_batch_noalloc(h, c_full, len(full), f_full))
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before
    _abi.check(lib, h, lib.rm_render_batch(h, c_full, len(full), ref_frames, _abi.RM_DEVICE))
    r.synchronize()
    for ref, got in zip(host(ref_bufs), host(b_full)):
        assert np.array_equal(ref["hit"], got["hit"])
        assert np.array_equal(ref["steps"], got["steps"])
        assert np.array_equal(ref["rgbd"].view(np.int32), got["rgbd"].view(np.int32))
        assert np.array_equal(ref["depth"].view(np.int32), got["depth"].view(np.int32))
    r.close()


def test_noalloc_rejects_batches_above_the_maximum():
    pytest.importorskip("torch")
    sc = syn.make_scene(5_000, n_boxes=2, seed=4)
    r = Renderer()
    r.set_cloud(sc.xyz, sc.rgb)
    r.build_index()
    r.compute_radii(0.1)
    n = 1025
    v = views_from_specs(syn.make_views(1, seed=5, boxes=sc.boxes, resolutions=[(8, 4)]))[0]
    cviews = (_abi.RmView * n)(*([v.to_c()] * n))
    frames = (_abi.RmFrame * n)()
    st = r._lib.rm_render_batch_noalloc(r._h, cviews, n, frames)
    assert st == _abi.RM_ERR_LIMIT
    assert b"1024" in r._lib.rm_last_error(r._h)
    r.close()
