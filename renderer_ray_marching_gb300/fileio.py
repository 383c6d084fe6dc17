"""Python access to the host file formats (``include/rmio.h``,
``lib/librm_io.so``): PLY clouds, the ``.kdtree.radii`` cache and the
per-view colour PNG / depth PNG / depth .npy outputs.  No GPU needed."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        _build.build()
        lib = ctypes.CDLL(_build.IOLIB)
        P, I32, I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        lib.rmio_last_error.restype = ctypes.c_char_p
        for name, args in {"rmio_ply_open": [ctypes.c_char_p, P], "rmio_ply_take": [P, P],
                           "rmio_ply_save": [ctypes.c_char_p, P, P, I64],
                           "rmio_radii_open": [ctypes.c_char_p, P], "rmio_radii_take": [P],
                           "rmio_radii_save": [ctypes.c_char_p, P, I64],
                           "rmio_write_frame": [ctypes.c_char_p, ctypes.c_char_p, I32, I32, P],
                           "rmio_json_mat4": [ctypes.c_char_p, P]}.items():
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = args
        _lib = lib
    return _lib


def _ok(rc):
    if rc != 0:
        raise RuntimeError(_lib.rmio_last_error().decode())


def load_ply(path: str):
    lib = _load()
    n = ctypes.c_int64()
    _ok(lib.rmio_ply_open(os.fsencode(path), ctypes.byref(n)))
    xyz = np.empty((n.value, 3), np.float32)
    rgb = np.empty((n.value, 3), np.uint8)
    _ok(lib.rmio_ply_take(xyz.ctypes.data, rgb.ctypes.data))
    return xyz, rgb


def save_ply(path: str, xyz, rgb) -> None:
    lib = _load()
    xyz = np.ascontiguousarray(xyz, np.float32)
    rgb = np.ascontiguousarray(rgb, np.uint8)
    _ok(lib.rmio_ply_save(os.fsencode(path), xyz.ctypes.data, rgb.ctypes.data, xyz.shape[0]))


def read_radii(path: str) -> np.ndarray:
    lib = _load()
    n = ctypes.c_int64()
    _ok(lib.rmio_radii_open(os.fsencode(path), ctypes.byref(n)))
    out = np.empty(n.value, np.float32)
    _ok(lib.rmio_radii_take(out.ctypes.data))
    return out


def write_radii(path: str, radii) -> None:
    lib = _load()
    r = np.ascontiguousarray(radii, np.float32)
    _ok(lib.rmio_radii_save(os.fsencode(path), r.ctypes.data, r.shape[0]))


def write_frame(colour_png: str, depth_png: str, rgbd) -> None:
    """rgbd: (H, W, 4) float32 render output, row 0 at the bottom."""
    lib = _load()
    a = np.ascontiguousarray(rgbd, np.float32)
    _ok(lib.rmio_write_frame(os.fsencode(colour_png), os.fsencode(depth_png), a.shape[1], a.shape[0],
                             a.ctypes.data))


def json_mat4(text: str) -> np.ndarray:
    lib = _load()
    out = np.empty(16, np.float32)
    _ok(lib.rmio_json_mat4(text.encode(), out.ctypes.data))
    return out
