"""The reference's GPU path restated (``ref_gpu.cu``): a timed baseline.

It is not the library and not the oracle: it restates what the reference
runs on its GPU -- the FLANN CUDA kd-tree and its exact k-NN search
(``third_party/flann/algorithms/kdtree_cuda_*``), and the render /
ray_march / distance_function kernel of ``src/ray_marching.cu`` with its
per-pixel global-memory result arrays -- so that the reference's GPU
execution can be timed on the GPU host, where the reference's own sources do
not travel.  ``bench.py`` times it beside the library and the tests check
that its hit maps equal the library's except where the two tie rules differ.

Built with nvcc's default floating-point flags (as the reference is), in
place, into ``_build/librefgpu.so``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "ref_gpu.cu")
_LIB = os.path.join(_HERE, "_build", "librefgpu.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    if (not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC)):
        return _LIB
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    tmp = _LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", _SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(build())
            P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
            lib.rg_create.restype = P
            lib.rg_create.argtypes = [P, I]
            lib.rg_error.restype = ctypes.c_char_p
            lib.rg_error.argtypes = [P]
            lib.rg_nodes.restype = I
            lib.rg_nodes.argtypes = [P]
            lib.rg_radii.restype = F
            lib.rg_radii.argtypes = [P, F, P, P]
            lib.rg_set_radii.restype = I
            lib.rg_set_radii.argtypes = [P, P]
            lib.rg_render.restype = F
            lib.rg_render.argtypes = [P, P, I, I, F, P, P]
            lib.rg_sqrt_loop_sample.restype = ctypes.c_double
            lib.rg_sqrt_loop_sample.argtypes = [P, I]
            lib.rg_destroy.argtypes = [P]
            _lib = lib
    return _lib


class RefGpu:
    """FLANN CUDA kd-tree over a cloud plus the reference's render kernel."""

    def __init__(self, xyz: np.ndarray):
        self._lib = _load()
        self.xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        self.n = self.xyz.shape[0]
        self._h = self._lib.rg_create(self.xyz.ctypes.data, self.n)
        err = self._lib.rg_error(self._h)
        if err:
            raise RuntimeError("ref_gpu: " + err.decode())

    def close(self):
        if self._h:
            self._lib.rg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, ms):
        if ms < 0:
            raise RuntimeError("ref_gpu: " + self._lib.rg_error(self._h).decode())
        return ms

    def radii(self, max_radius: float = 0.1):
        """(radii, second-neighbour index, kernel ms); the render radii become
        min(r, max_radius)."""
        r = np.empty(self.n, np.float32)
        nn = np.empty(self.n, np.int32)
        ms = self._check(self._lib.rg_radii(self._h, max_radius, r.ctypes.data, nn.ctypes.data))
        return r, nn, ms

    def sqrt_loop_seconds_per_point(self, count: int = 20000) -> float:
        """Seconds per point of the reference's host sqrt loop over device
        elements (two synchronous 4-byte copies per point), timed on `count`
        points."""
        secs = self._lib.rg_sqrt_loop_sample(self._h, int(count))
        if secs < 0:
            raise RuntimeError("ref_gpu: sqrt loop sample failed")
        return secs / min(int(count), self.n)

    def set_radii(self, radii_clamped: np.ndarray):
        r = np.ascontiguousarray(radii_clamped, np.float32)
        if self._lib.rg_set_radii(self._h, r.ctypes.data) != 0:
            raise RuntimeError("ref_gpu: " + self._lib.rg_error(self._h).decode())

    def render_into(self, cam2world_colmajor, width: int, height: int, fov: float, hit_ptr: int, depth_ptr: int):
        """One view into device arrays (hit int32, depth float32, W*H each);
        returns the kernel time in ms."""
        m = np.ascontiguousarray(cam2world_colmajor, np.float32).reshape(16)
        return self._check(self._lib.rg_render(self._h, m.ctypes.data, int(width), int(height), float(fov),
                                               hit_ptr, depth_ptr))
