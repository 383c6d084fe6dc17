"""The marcher's neighbour set (``rm::KSet``) against a sort, on the GPU.

Each step of the marcher keeps its 10 nearest points in ``KSet``: a common
insertion that orders by d2 alone, an ordered insertion (by d2, then cloud
index) when an exact tie sits at the set's boundary, and ``order()``, which
sorts runs of equal d2 by cloud index before the set is read.  Equal d2 is
rare in real clouds except for duplicated points, so the parity tests meet
these paths only through the duplicate-point cloud.  This test drives them
directly: ``tests/kset_probe.cu`` runs the device code on 65,536 sequences
of candidates whose d2 values are drawn from a few levels (many exact ties),
each starting from placeholders at a bound as a step does, with the walk's
filter (a candidate is offered only when its d2 is <= the current bound).
The result must be exactly the 10 smallest (d2, cloud index) among the
candidates within the bound, in that order, padded with placeholders --
the ordering of ``src/ray_marching.cu:280-290`` over FLANN's sorted result
set.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "kset_probe.cu")
OUT = os.path.join(HERE, "_build", "libkset_probe.so")
K = 10


def _nvcc():
    p = "/usr/local/cuda/bin/nvcc"
    return p if os.path.exists(p) else "nvcc"


@pytest.fixture(scope="module")
def probe():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "renderer_ray_marching_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    lib = ctypes.CDLL(OUT)
    P = ctypes.c_void_p
    lib.kset_run.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int, P, P]
    lib.kset_run.restype = ctypes.c_int
    return lib, torch


def _cases(seed, seqs, length, n_points):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_points).astype(np.int32)
    levels = rng.choice([3, 6, 12, 1000], size=seqs)
    d2 = (rng.integers(0, 1 << 20, size=(seqs, length)) % (levels[:, None] + 1)).astype(np.float32) * np.float32(1e-6)
    pos = np.stack([rng.choice(n_points, size=length, replace=False) for _ in range(seqs)]).astype(np.int32)
    counts = rng.integers(0, length + 1, size=seqs)
    pos[np.arange(length)[None, :] >= counts[:, None]] = -1  # ragged sequences
    # bounds: none (+inf), between levels, and exactly on a level (ties with the bound)
    kind = rng.integers(0, 3, size=seqs)
    lvl = rng.integers(0, levels + 1).astype(np.float32) * np.float32(1e-6)
    bound = np.where(kind == 0, np.float32(np.inf),
                     np.where(kind == 1, lvl + np.float32(0.5e-6), lvl)).astype(np.float32)
    return perm, d2, pos, bound


def _expected(perm, d2, pos, bound):
    seqs = d2.shape[0]
    exp_d = np.empty((seqs, K), np.float32)
    exp_s = np.full((seqs, K), -1, np.int32)
    for t in range(seqs):
        ok = (pos[t] >= 0) & (d2[t] <= bound[t])
        dd, ss = d2[t][ok], pos[t][ok]
        order = np.lexsort((perm[ss], dd))[:K]
        m = order.size
        exp_d[t, :m] = dd[order]
        exp_d[t, m:] = bound[t]
        exp_s[t, :m] = ss[order]
    return exp_d, exp_s


@pytest.mark.parametrize("seed,length", [(1, 24), (2, 64), (3, 200)])
def test_neighbour_set_equals_sort_by_distance_then_cloud_index(probe, seed, length):
    lib, torch = probe
    seqs, n_points = 65536 if length <= 64 else 8192, 4096
    perm, d2, pos, bound = _cases(seed, seqs, length, n_points)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t_d2, t_pos, t_bound, t_perm = dev(d2), dev(pos), dev(bound), dev(perm)
    out_d = torch.empty((seqs, K), dtype=torch.float32, device="cuda")
    out_s = torch.empty((seqs, K), dtype=torch.int32, device="cuda")
    assert lib.kset_run(t_d2.data_ptr(), t_pos.data_ptr(), t_bound.data_ptr(), t_perm.data_ptr(), seqs, length,
                        out_d.data_ptr(), out_s.data_ptr()) == 0
    got_d, got_s = out_d.cpu().numpy(), out_s.cpu().numpy()
    exp_d, exp_s = _expected(perm, d2, pos, bound)
    bad = np.nonzero((got_s != exp_s).any(axis=1) | (got_d.view(np.int32) != exp_d.view(np.int32)).any(axis=1))[0]
    assert bad.size == 0, "%d of %d sequences differ; first %d: got %s / %s, expected %s / %s" % (
        bad.size, seqs, bad[0], got_s[bad[0]], got_d[bad[0]], exp_s[bad[0]], exp_d[bad[0]])
    # the cases do reach the tie paths: many sequences hold equal d2 inside their final set
    with np.errstate(invalid="ignore"):
        ties = (np.diff(exp_d, axis=1) == 0) & (exp_s[:, 1:] >= 0)
    assert ties.any(axis=1).mean() > 0.3
