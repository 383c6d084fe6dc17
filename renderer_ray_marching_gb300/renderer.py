"""Python front end of the C ABI.

``Renderer`` holds one ``rm_ctx`` and mirrors the operations of the
reference's two in-process classes: ``kdtree::KDTreeFlann``
(``src/kdtree/kdtree_flann.h:15-43``: Build, Search with a kNN parameter)
and ``PointcloudRayMarcher`` (``src/ray_marching.h:11-44``:
construction from vertices/colours/radii/tree, render_to_texture).
Arrays may be numpy arrays (host memory; the library copies) or CUDA torch
tensors (device memory; the library works in place on its stream).
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import _abi

try:  # torch is only needed for device-resident buffers
    import torch
except Exception:  # pragma: no cover - torch is present in this project's images
    torch = None


@dataclasses.dataclass
class View:
    """One camera: column-major cam-to-world (OpenGL convention), image size
    and horizontal field of view in radians (render_to_texture's arguments,
    src/ray_marching.cu:93-96)."""
    cam2world: np.ndarray
    width: int
    height: int
    fov: float

    def to_c(self) -> _abi.RmView:
        v = _abi.RmView()
        m = np.ascontiguousarray(self.cam2world, np.float32).reshape(16)
        for i in range(16):
            v.cam2world[i] = float(m[i])
        v.width = int(self.width)
        v.height = int(self.height)
        v.fov = float(np.float32(self.fov))
        return v

    @property
    def pixels(self) -> int:
        return int(self.width) * int(self.height)


def views_from_specs(specs) -> list[View]:
    from .synthetic import view_params
    out = []
    for s in specs:
        m, w, h, fov = view_params(s)
        out.append(View(m, w, h, float(fov)))
    return out


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def _loc_ptr(a, dtype):
    """(location, pointer, keep-alive) of an array argument."""
    if a is None:
        return None, None, None
    if _is_torch(a):
        if not a.is_cuda:
            a = a.numpy()
        else:
            want = {np.float32: torch.float32, np.int32: torch.int32, np.uint8: torch.uint8}[dtype]
            if a.dtype != want or not a.is_contiguous():
                a = a.to(want).contiguous()
            return _abi.RM_DEVICE, a.data_ptr(), a
    arr = np.ascontiguousarray(a, dtype=dtype)
    return _abi.RM_HOST, arr.ctypes.data, arr


class Renderer:
    """One renderer context on one CUDA device."""

    def __init__(self, leaf_size: int = 16, device: int = 0, stream: int | None = None):
        self._lib = _abi.load()
        cfg = _abi.RmConfig()
        self._lib.rm_config_default(ctypes.byref(cfg))
        cfg.leaf_size = leaf_size
        cfg.device = device
        cfg.stream = stream
        h = ctypes.c_void_p()
        st = self._lib.rm_ctx_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != _abi.RM_OK:
            raise _abi.RmError(st, "rm_ctx_create failed (is a CUDA device present?)")
        self._h = h
        self.device = device
        self.n = 0

    # -- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.rm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        _abi.check(self._lib, self._h, st)

    def synchronize(self):
        self._check(self._lib.rm_synchronize(self._h))

    # -- cloud, index, radii -------------------------------------------
    def set_cloud(self, xyz, rgb=None):
        """Upload points (N x 3 or N x stride float32) and uint8 colours."""
        if _is_torch(xyz) and xyz.is_cuda:
            x = xyz.to(torch.float32).contiguous()
            n, stride = x.shape[0], (x.shape[1] if x.dim() == 2 else 3)
            c = None
            if rgb is not None:
                c = rgb.to(device=x.device, dtype=torch.uint8).contiguous()
            self._check(self._lib.rm_cloud_set(self._h, x.data_ptr(), stride,
                                               c.data_ptr() if c is not None else None, n,
                                               _abi.RM_DEVICE))
        else:
            x = np.ascontiguousarray(xyz, np.float32)
            n, stride = x.shape[0], (x.shape[1] if x.ndim == 2 else 3)
            c = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
            self._check(self._lib.rm_cloud_set(self._h, x.ctypes.data, stride,
                                               c.ctypes.data if c is not None else None, n,
                                               _abi.RM_HOST))
        self.n = int(n)

    def build_index(self):
        self._check(self._lib.rm_index_build(self._h))

    def compute_radii(self, max_radius: float = 0.1, device: bool = False):
        """Unclamped radii and second-neighbour index, cloud order; the context
        keeps min(r, max_radius) for rendering."""
        if device:
            r = torch.empty(self.n, dtype=torch.float32, device="cuda:%d" % self.device)
            nn = torch.empty(self.n, dtype=torch.int32, device=r.device)
            self._check(self._lib.rm_radii_compute(self._h, max_radius, r.data_ptr(), nn.data_ptr(),
                                                   _abi.RM_DEVICE))
            self.synchronize()
            return r, nn
        r = np.empty(self.n, np.float32)
        nn = np.empty(self.n, np.int32)
        self._check(self._lib.rm_radii_compute(self._h, max_radius, r.ctypes.data, nn.ctypes.data,
                                               _abi.RM_HOST))
        return r, nn

    def set_radii(self, radii, max_radius: float = 0.1):
        loc, ptr, keep = _loc_ptr(radii, np.float32)
        n = keep.shape[0] if keep is not None else 0
        self._check(self._lib.rm_radii_set(self._h, ptr, n, max_radius, loc))
        del keep

    def knn(self, queries, k: int):
        loc, ptr, keep = _loc_ptr(queries, np.float32)
        m = keep.shape[0]
        stride = keep.shape[1] if keep.ndim == 2 else 3
        if loc == _abi.RM_DEVICE:
            idx = torch.empty((m, k), dtype=torch.int32, device=keep.device)
            d2 = torch.empty((m, k), dtype=torch.float32, device=keep.device)
            self._check(self._lib.rm_knn(self._h, ptr, stride, m, k, idx.data_ptr(), d2.data_ptr(), loc))
            self.synchronize()
            return idx, d2
        idx = np.empty((m, k), np.int32)
        d2 = np.empty((m, k), np.float32)
        self._check(self._lib.rm_knn(self._h, ptr, stride, m, k, idx.ctypes.data, d2.ctypes.data, loc))
        return idx, d2

    # -- views ------------------------------------------------------------
    def view_pane(self, views) -> np.ndarray:
        arr = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        out = np.empty(len(views), np.float32)
        self._check(self._lib.rm_view_pane(self._h, arr, len(views), out.ctypes.data))
        return out

    # -- rendering ----------------------------------------------------------
    _FIELDS = (("rgbd", 4, np.float32), ("hit", 1, np.int32), ("depth", 1, np.float32),
               ("steps", 1, np.int32))

    def _alloc_frame(self, view: View, outputs, device: bool):
        bufs = {}
        fr = _abi.RmFrame()
        for name, ch, dt in self._FIELDS:
            if name not in outputs:
                continue
            shape = (view.height, view.width, ch) if ch > 1 else (view.height, view.width)
            if device:
                tdt = torch.float32 if dt == np.float32 else torch.int32
                b = torch.empty(shape, dtype=tdt, device="cuda:%d" % self.device)
                setattr(fr, name, b.data_ptr())
            else:
                b = np.empty(shape, dt)
                setattr(fr, name, b.ctypes.data)
            bufs[name] = b
        return fr, bufs

    def render(self, view: View, outputs=("rgbd", "hit", "depth"), device: bool = False) -> dict:
        """Plain form: one view, one launch.  Images have row 0 at the bottom."""
        fr, bufs = self._alloc_frame(view, outputs, device)
        v = view.to_c()
        self._check(self._lib.rm_render(self._h, ctypes.byref(v), ctypes.byref(fr),
                                        _abi.RM_DEVICE if device else _abi.RM_HOST))
        if device:
            self.synchronize()
        return bufs

    def render_into(self, view: View, frame: dict, device: bool = True):
        """Plain render into caller buffers (dict of name -> tensor/array)."""
        fr = _abi.RmFrame()
        for name, _, _ in self._FIELDS:
            if name in frame:
                b = frame[name]
                setattr(fr, name, b.data_ptr() if _is_torch(b) else b.ctypes.data)
        v = view.to_c()
        self._check(self._lib.rm_render(self._h, ctypes.byref(v), ctypes.byref(fr),
                                        _abi.RM_DEVICE if device else _abi.RM_HOST))

    def render_batch(self, views, outputs=("rgbd", "hit", "depth"), device: bool = True) -> list:
        """Batched form: all views in one persistent, graph-replayed launch."""
        frames = (_abi.RmFrame * len(views))()
        bufs = []
        for i, v in enumerate(views):
            fr, b = self._alloc_frame(v, outputs, device)
            frames[i] = fr
            bufs.append(b)
        self.render_batch_into(views, frames, device)
        if device:
            self.synchronize()
        return bufs

    def render_batch_into(self, views, frames, device: bool = True, cviews=None):
        if cviews is None:
            cviews = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        self._check(self._lib.rm_render_batch(self._h, cviews, len(views), frames,
                                              _abi.RM_DEVICE if device else _abi.RM_HOST))

    def set_launch(self, tile_w=8, tile_h=4, rays_per_lane=1, ctas_per_sm=8, search=1):
        L = _abi.RmLaunch(tile_w, tile_h, rays_per_lane, ctas_per_sm, search)
        self._check(self._lib.rm_set_launch(self._h, ctypes.byref(L)))

    def get_launch(self) -> dict:
        L = _abi.RmLaunch()
        self._check(self._lib.rm_get_launch(self._h, ctypes.byref(L)))
        return {"tile_w": L.tile_w, "tile_h": L.tile_h, "rays_per_lane": L.rays_per_lane,
                "ctas_per_sm": L.ctas_per_sm, "search": L.search}

    def autotune(self, views) -> dict:
        arr = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        L = _abi.RmLaunch()
        leaf = ctypes.c_int32()
        ms = ctypes.c_float()
        self._check(self._lib.rm_autotune(self._h, arr, len(views), ctypes.byref(L), ctypes.byref(leaf),
                                          ctypes.byref(ms)))
        return {"tile_w": L.tile_w, "tile_h": L.tile_h, "rays_per_lane": L.rays_per_lane,
                "ctas_per_sm": L.ctas_per_sm, "search": L.search,
                "leaf_size": leaf.value, "ms": round(ms.value, 3)}

    def stats(self) -> dict:
        s = _abi.RmStats()
        self._check(self._lib.rm_get_stats(self._h, ctypes.byref(s)))
        return {"rays": s.rays, "steps": s.steps, "hits": s.hits, "packet_steps": s.packet_steps,
                "search_errors": s.search_errors,
                "solo_steps": s.solo_steps, "packet_leaves": s.packet_leaves, "packet_nodes": s.packet_nodes,
                "warp_steps": s.warp_steps, "split_steps": s.split_steps, "kernel_ms": s.kernel_ms,
                "queue_spills": s.queue_spills, "dfs_walks": s.dfs_walks}

    # -- backward -------------------------------------------------------------
    def backward(self, views, dl_drgb, dl_ddepth, hit, g_rgb, g_xyz, g_radius):
        """Accumulate first-hit gradients (see rm_backward in include/rm.h).
        All arrays torch CUDA tensors (device) or all numpy (host)."""
        arr = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        dev = _is_torch(dl_drgb) and dl_drgb.is_cuda
        loc = _abi.RM_DEVICE if dev else _abi.RM_HOST

        def p(a, dt):
            if dev:
                return a.data_ptr()
            assert isinstance(a, np.ndarray) and a.dtype == dt and a.flags.c_contiguous
            return a.ctypes.data

        self._check(self._lib.rm_backward(self._h, arr, len(views), p(dl_drgb, np.float32),
                                          p(dl_ddepth, np.float32), p(hit, np.int32),
                                          p(g_rgb, np.float32), p(g_xyz, np.float32),
                                          p(g_radius, np.float32), loc))
