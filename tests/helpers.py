"""Shared test helpers: exact brute-force kNN and small scene builders."""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.fmaf.restype = ctypes.c_float
_libm.fmaf.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]


def fmaf(a, b, c):
    """Correctly rounded float32 fused multiply-add (C's fmaf), elementwise."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    c = np.asarray(c, np.float32)
    a, b, c = np.broadcast_arrays(a, b, c)
    out = np.empty(a.shape, np.float32)
    fa, fb, fc, fo = a.ravel(), b.ravel(), c.ravel(), out.reshape(-1)
    for i in range(fo.size):
        fo[i] = _libm.fmaf(float(fa[i]), float(fb[i]), float(fc[i]))
    return out


def d2_exact(c: np.ndarray, q: np.ndarray) -> np.ndarray:
    """fmaf(dz, dz, fmaf(dx, dx, dy*dy)) for all points c against one query q."""
    d = (c.astype(np.float32) - q.astype(np.float32)).astype(np.float32)
    yy = (d[:, 1] * d[:, 1]).astype(np.float32)
    t = fmaf(d[:, 0], d[:, 0], yy)
    return fmaf(d[:, 2], d[:, 2], t)


def brute_knn(xyz: np.ndarray, q: np.ndarray, k: int):
    n = xyz.shape[0]
    idx = np.full((q.shape[0], k), -1, np.int32)
    d2 = np.full((q.shape[0], k), np.inf, np.float32)
    for i in range(q.shape[0]):
        d = d2_exact(xyz, q[i])
        order = np.lexsort((np.arange(n), d))[:k]
        idx[i, :len(order)] = order
        d2[i, :len(order)] = d[order]
    return idx, d2


def f32_ulp_close(a, b, ulps: int) -> np.ndarray:
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b) <= ulps


def d2_fast(c: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Vectorised fmaf(dz, dz, fmaf(dx, dx, dy*dy)): each fma is one exact
    float64 product plus one addition, rounded to float32.  The float64 sum
    is exact unless the addends' exponents are far apart, and a double
    rounding would need the float64 result to sit exactly on a float32
    midpoint; brute_knn (true fmaf) is the slow exact fallback."""
    d = (c.astype(np.float32) - q.astype(np.float32)).astype(np.float32)
    d64 = d.astype(np.float64)
    yy = (d[:, 1] * d[:, 1]).astype(np.float32).astype(np.float64)
    t = (d64[:, 0] * d64[:, 0] + yy).astype(np.float32).astype(np.float64)
    return (d64[:, 2] * d64[:, 2] + t).astype(np.float32)


def brute_march(xyz, radii, o, d, t_near, t_far, max_steps=128, min_dist=np.float32(0.001)):
    """The reference marcher loop (src/ray_marching.cu:202-292) with a
    brute-force 10-NN: returns (hit, depth, steps)."""
    n = xyz.shape[0]
    t = np.float32(t_near)
    idx = np.arange(n)
    for i in range(max_steps):
        p = np.array([np.float32(fmaf(d[a], t, o[a])) for a in range(3)], np.float32)
        dd = d2_fast(xyz, p)
        # the 10 nearest in (d2, index) order, exact under ties: every point
        # tied with the 10th distance is a candidate before the final sort
        if n > 10:
            kth = np.partition(dd, 9)[9]
            part = np.nonzero(dd <= kth)[0]
        else:
            part = idx
        order = part[np.lexsort((part, dd[part]))][:10]
        best, bi = np.float32(np.inf), 0
        for j in order:
            v = np.float32(np.sqrt(dd[j], dtype=np.float32) - radii[j])
            if v < best:
                best, bi = v, int(j)
        t = np.float32(t + best)
        if best < min_dist:
            return bi, t, i + 1
        if t > t_far:
            return -1, np.float32(0), i + 1
    return -1, np.float32(0), max_steps
