"""ctypes binding of ``include/rm.h`` (the C ABI of ``lib/librm_gb300.so``).

This is the Python side of the drop-in boundary: the structs and function
prototypes below mirror the header one to one.  There is no fallback: if
the library cannot be built or loaded, or no CUDA device is present, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

RM_OK, RM_ERR_INVALID, RM_ERR_STATE, RM_ERR_CUDA, RM_ERR_OOM, RM_ERR_LIMIT, RM_ERR_KERNEL = range(7)
RM_HOST, RM_DEVICE = 0, 1
RM_NOALLOC_MAX_VIEWS = 1024  # include/rm.h
STATUS_NAMES = {0: "RM_OK", 1: "RM_ERR_INVALID", 2: "RM_ERR_STATE", 3: "RM_ERR_CUDA",
                4: "RM_ERR_OOM", 5: "RM_ERR_LIMIT", 6: "RM_ERR_KERNEL"}

# Every symbol include/rm.h declares (checked by the CPU tests).
EXPORTS = [
    "rm_config_default", "rm_ctx_create", "rm_ctx_destroy", "rm_last_error", "rm_synchronize",
    "rm_cloud_set", "rm_index_build", "rm_knn", "rm_radii_compute", "rm_radii_set",
    "rm_view_pane", "rm_render", "rm_render_batch", "rm_set_launch", "rm_get_launch",
    "rm_autotune", "rm_get_stats", "rm_backward", "rm_cloud_size", "rm_render_batch_noalloc",
]


class RmConfig(ctypes.Structure):
    _fields_ = [("zfar", ctypes.c_float), ("znear", ctypes.c_float), ("max_steps", ctypes.c_int32),
                ("min_dist", ctypes.c_float), ("knn", ctypes.c_int32), ("leaf_size", ctypes.c_int32),
                ("device", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class RmView(ctypes.Structure):
    _fields_ = [("cam2world", ctypes.c_float * 16), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("fov", ctypes.c_float)]


class RmFrame(ctypes.Structure):
    _fields_ = [("rgbd", ctypes.c_void_p), ("hit", ctypes.c_void_p), ("depth", ctypes.c_void_p),
                ("steps", ctypes.c_void_p)]


class RmStats(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_int64), ("steps", ctypes.c_int64), ("hits", ctypes.c_int64),
                ("packet_steps", ctypes.c_int64), ("solo_steps", ctypes.c_int64),
                ("packet_leaves", ctypes.c_int64), ("packet_nodes", ctypes.c_int64),
                ("warp_steps", ctypes.c_int64), ("split_steps", ctypes.c_int64),
                ("search_errors", ctypes.c_int64), ("kernel_ms", ctypes.c_float),
                ("queue_spills", ctypes.c_int64), ("dfs_walks", ctypes.c_int64)]


class RmLaunch(ctypes.Structure):
    _fields_ = [("tile_w", ctypes.c_int32), ("tile_h", ctypes.c_int32),
                ("rays_per_lane", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("search", ctypes.c_int32)]


class RmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the shared library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build_if_missing else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("renderer library not built: %s" % path)
        lib = ctypes.CDLL(path)
        P, I32, I64, F = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
        sig = {
            "rm_config_default": (None, [P]),
            "rm_ctx_create": (I32, [P, P]),
            "rm_ctx_destroy": (None, [P]),
            "rm_last_error": (ctypes.c_char_p, [P]),
            "rm_synchronize": (I32, [P]),
            "rm_cloud_set": (I32, [P, P, I32, P, I64, I32]),
            "rm_index_build": (I32, [P]),
            "rm_knn": (I32, [P, P, I32, I64, I32, P, P, I32]),
            "rm_radii_compute": (I32, [P, F, P, P, I32]),
            "rm_radii_set": (I32, [P, P, I64, F, I32]),
            "rm_view_pane": (I32, [P, P, I32, P]),
            "rm_render": (I32, [P, P, P, I32]),
            "rm_render_batch": (I32, [P, P, I32, P, I32]),
            "rm_set_launch": (I32, [P, P]),
            "rm_get_launch": (I32, [P, P]),
            "rm_autotune": (I32, [P, P, I32, P, P, P]),
            "rm_get_stats": (I32, [P, P]),
            "rm_backward": (I32, [P, P, I32, P, P, P, P, P, P, I32]),
            "rm_cloud_size": (I64, [P]),
            "rm_render_batch_noalloc": (I32, [P, P, I32, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(lib, ctx, status: int) -> None:
    if status != RM_OK:
        msg = lib.rm_last_error(ctx)
        raise RmError(status, msg.decode() if msg else "")
