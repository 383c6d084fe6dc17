"""CPU oracle for the renderer hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package.  It is the checker, never the product: the
CUDA library in ``renderer_ray_marching_gb300`` never calls into it.

The C code (``rm_oracle.c``) restates the reference's radii precompute
(``main.cu:102-149``), its ray generation and sphere-tracing loop
(``src/ray_marching.cu:63-91, 202-228``) and its 10-nearest-centre distance
function (``src/ray_marching.cu:260-292``) with every rounding step written
out, so the same bits come out on x86-64 and aarch64.  It is pinned against
FLANN's own CPU kd-tree (the reference's vendored ``third_party/flann``)
through the fixtures in ``tests/golden/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "librm_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc, -ffp-contract=off, OpenMP)."""
    src = os.path.join(_HERE, "rm_oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(os.path.join(_HERE, "rm_oracle.h"))):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class View(ctypes.Structure):
    _fields_ = [("cam2world", ctypes.c_float * 16), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("pane", ctypes.c_float)]


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        lib.rmo_index_build.restype = P
        lib.rmo_index_build.argtypes = [P, ctypes.c_int64]
        lib.rmo_index_free.argtypes = [P]
        lib.rmo_knn.argtypes = [P, P, ctypes.c_int64, ctypes.c_int, P, P, ctypes.c_int]
        lib.rmo_radii.argtypes = [P, ctypes.c_float, P, P, ctypes.c_int]
        lib.rmo_render.argtypes = [P, P, P, P, ctypes.c_int64, P, P, P, ctypes.c_int]
        lib.rmo_distance.restype = ctypes.c_float
        lib.rmo_distance.argtypes = [P, P, P, P]
        lib.rmo_ray.argtypes = [P, ctypes.c_int32, ctypes.c_int32, P, P, P, P]
        lib.rmo_sphere_depth.restype = ctypes.c_double
        lib.rmo_sphere_depth.argtypes = [P, P, P, ctypes.c_double, P, P, P]
        _lib = lib
        return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_view(cam2world_colmajor, width: int, height: int, pane: float) -> View:
    v = View()
    m = np.ascontiguousarray(cam2world_colmajor, dtype=np.float32).reshape(16)
    for i in range(16):
        v.cam2world[i] = float(m[i])
    v.width = int(width)
    v.height = int(height)
    v.pane = float(np.float32(pane))
    return v


class Index:
    """Exact kNN index over float32 xyz points (original order kept)."""

    def __init__(self, xyz: np.ndarray):
        self._lib = _load()
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        self.n = self.xyz.shape[0]
        self._h = self._lib.rmo_index_build(_ptr(self.xyz), self.n)

    def close(self):
        if self._h:
            self._lib.rmo_index_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def knn(self, q: np.ndarray, k: int, threads: int = 0):
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, 3)
        idx = np.empty((q.shape[0], k), np.int32)
        d2 = np.empty((q.shape[0], k), np.float32)
        self._lib.rmo_knn(self._h, _ptr(q), q.shape[0], k, _ptr(idx), _ptr(d2), threads)
        return idx, d2

    def radii(self, max_radius: float = 0.0, threads: int = 0):
        r = np.empty(self.n, np.float32)
        nn = np.empty(self.n, np.int32)
        self._lib.rmo_radii(self._h, ctypes.c_float(max_radius), _ptr(r), _ptr(nn), threads)
        return r, nn

    def render(self, radii: np.ndarray, view: View, pixels=None, threads: int = 0):
        radii = np.ascontiguousarray(radii, dtype=np.float32)
        if pixels is None:
            pixels = np.arange(view.width * view.height, dtype=np.int64)
        pixels = np.ascontiguousarray(pixels, dtype=np.int64)
        hit = np.empty(pixels.shape[0], np.int32)
        depth = np.empty(pixels.shape[0], np.float32)
        steps = np.empty(pixels.shape[0], np.int32)
        self._lib.rmo_render(self._h, _ptr(radii), ctypes.byref(view), _ptr(pixels),
                             pixels.shape[0], _ptr(hit), _ptr(depth), _ptr(steps), threads)
        return hit, depth, steps

    def distance(self, radii: np.ndarray, p):
        radii = np.ascontiguousarray(radii, dtype=np.float32)
        p = np.ascontiguousarray(p, dtype=np.float32).reshape(3)
        idx = ctypes.c_int32(0)
        s = self._lib.rmo_distance(self._h, _ptr(radii), _ptr(p), ctypes.byref(idx))
        return float(s), int(idx.value)


def ray(view: View, x: int, y: int):
    lib = _load()
    o = np.empty(3, np.float32)
    d = np.empty(3, np.float32)
    tn = ctypes.c_float()
    tf = ctypes.c_float()
    lib.rmo_ray(ctypes.byref(view), x, y, _ptr(o), _ptr(d), ctypes.byref(tn), ctypes.byref(tf))
    return o, d, np.float32(tn.value), np.float32(tf.value)


def sphere_depth(o, d, c, r: float):
    """FP64 analytic entry distance and its gradient w.r.t. centre and radius."""
    lib = _load()
    o = np.ascontiguousarray(o, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    t = ctypes.c_double()
    gc = np.empty(3, np.float64)
    gr = ctypes.c_double()
    disc = lib.rmo_sphere_depth(_ptr(o), _ptr(d), _ptr(c), float(r), ctypes.byref(t), _ptr(gc),
                                ctypes.byref(gr))
    return t.value, gc, gr.value, disc
