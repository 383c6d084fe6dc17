"""The floating-point contract behind bit-exact parity, pinned on the GPU.

The reference's kernels are plain CUDA C++ compiled with nvcc's defaults, so
nvcc decides where a multiply feeding an add becomes one fused multiply-add.
The library writes every rounding step out with _rn intrinsics instead
(``csrc/rm_device.cuh``), and the CPU oracle copies those steps.  This test
builds ``tests/fp_contract.cu`` with nvcc's default contraction (no
``--fmad=false``, no fast-math) and checks, on 2.2e7 random and adversarial
inputs, that the reference's own source expressions and the library's
functions give the same bits:

- squared distance ``dot(a - b, a - b)`` over float4 with w = 0
  (``third_party/flann/algorithms/kdtree_cuda_3d_index.cu:186-192``,
  ``util/cutil_math.h:596-599, 1127-1130``) against ``rm::d2_point``;
- the step position ``ray_origin + ray_dir * t`` (``src/ray_marching.cu:216``);
- the float3 dot of the plane distances (``src/ray_marching.cu:78-79``);
- the step value ``sqrtf(D) - R`` (``src/ray_marching.cu:285``);
- the whole ray set-up of ``src/ray_marching.cu:71-79`` with glm 0.9.9.8's
  published mat4*vec4, dot and normalize, against ``rm::make_ray``.

The nvcc here is the one that builds the library; the reference's own
binary came from an older nvcc, whose contraction is not pinned by this test.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "fp_contract.cu")
OUT = os.path.join(HERE, "_build", "libfp_contract.so")


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
    # nvcc's defaults on purpose: -fmad=true, IEEE division and square root
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "renderer_ray_marching_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    lib = ctypes.CDLL(OUT)
    P, I64 = ctypes.c_void_p, ctypes.c_int64
    lib.fpc_d2.argtypes = [P, P, I64, P, P]
    lib.fpc_step.argtypes = [P, P, P, I64, P, P]
    lib.fpc_dot3.argtypes = [P, P, I64, P, P]
    lib.fpc_stepval.argtypes = [P, P, I64, P, P]
    lib.fpc_ray.argtypes = [P, P, P, P, I64, P, P]
    return lib, torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _same_bits(ref, lib, what):
    r = ref.cpu().numpy().view(np.int32).reshape(-1)
    g = lib.cpu().numpy().view(np.int32).reshape(-1)
    bad = np.nonzero(r != g)[0]
    assert bad.size == 0, "%s: %d of %d differ, first at %s (ref %r, lib %r)" % (
        what, bad.size, r.size, bad[:5], r.view(np.float32)[bad[:5]], g.view(np.float32)[bad[:5]])


def _d2_cases(rng):
    f = np.float32
    n = 2_000_000
    cases = []
    # scene scale, far queries
    c = rng.uniform(-10, 10, (n, 3))
    cases.append((c, rng.uniform(-10, 10, (n, 3))))
    # cancellation: query within a millimetre of the point
    c = rng.uniform(0, 8, (n, 3))
    cases.append((c, c + rng.normal(0, 1e-3, (n, 3))))
    # neighbourhood of a surface point, room scale
    c = rng.uniform(0, 8, (n, 3))
    cases.append((c, c + rng.normal(0, 0.05, (n, 3))))
    # a cloud far from the origin (coarse float spacing)
    c = 1e4 + rng.uniform(-1, 1, (n, 3))
    cases.append((c, c + rng.normal(0, 1e-2, (n, 3))))
    # subnormal products and sums
    m = 1_000_000
    cases.append((rng.normal(0, 1e-19, (m, 3)), rng.normal(0, 1e-19, (m, 3))))
    # axis gaps of very different magnitude
    g = np.stack([rng.normal(0, 1, m), rng.normal(0, 1e-4, m), rng.normal(0, 1e-8, m)], 1)
    c = rng.uniform(0, 8, (m, 3))
    cases.append((c, c + g))
    cs = np.concatenate([x[0] for x in cases]).astype(f)
    qs = np.concatenate([x[1] for x in cases]).astype(f)
    pad = np.zeros((cs.shape[0], 1), f)
    return np.concatenate([cs, pad], 1), np.concatenate([qs, pad], 1)


def test_squared_distance_contracts_as_the_library_writes_it(probe):
    lib, torch = probe
    c, q = _d2_cases(np.random.default_rng(1))
    assert c.shape[0] >= 10_000_000
    cd, qd = _dev(torch, c), _dev(torch, q)
    ref = torch.empty(c.shape[0], dtype=torch.float32, device="cuda")
    got = torch.empty_like(ref)
    assert lib.fpc_d2(cd.data_ptr(), qd.data_ptr(), c.shape[0], ref.data_ptr(), got.data_ptr()) == 0
    _same_bits(ref, got, "d2")


def test_step_position_dot_and_step_value(probe):
    lib, torch = probe
    rng = np.random.default_rng(2)
    n = 4_000_000
    o = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    o[: n // 4] += np.float32(1e4)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t = np.concatenate([rng.uniform(0.1, 100, n // 2), 10.0 ** rng.uniform(-6, 2, n - n // 2)]).astype(np.float32)
    od, dd, td = _dev(torch, o), _dev(torch, d), _dev(torch, t)
    ref = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    got = torch.empty_like(ref)
    assert lib.fpc_step(od.data_ptr(), dd.data_ptr(), td.data_ptr(), n, ref.data_ptr(), got.data_ptr()) == 0
    _same_bits(ref, got, "o + d t")
    # float3 dot: unit vectors, and mixed magnitudes
    a = rng.normal(size=(n, 3)).astype(np.float32)
    b = d.copy()
    a[n // 2:] *= 10.0 ** rng.uniform(-20, 20, (n - n // 2, 3)).astype(np.float32)
    ad, bd = _dev(torch, a), _dev(torch, b)
    ref1 = torch.empty(n, dtype=torch.float32, device="cuda")
    got1 = torch.empty_like(ref1)
    assert lib.fpc_dot3(ad.data_ptr(), bd.data_ptr(), n, ref1.data_ptr(), got1.data_ptr()) == 0
    _same_bits(ref1, got1, "dot3")
    # step value sqrtf(D) - R
    m = 2_000_000
    d2 = (10.0 ** rng.uniform(-12, 4, m)).astype(np.float32)
    r = rng.uniform(0, 0.1, m).astype(np.float32)
    d2d, rd = _dev(torch, d2), _dev(torch, r)
    ref2 = torch.empty(m, dtype=torch.float32, device="cuda")
    got2 = torch.empty_like(ref2)
    assert lib.fpc_stepval(d2d.data_ptr(), rd.data_ptr(), m, ref2.data_ptr(), got2.data_ptr()) == 0
    _same_bits(ref2, got2, "sqrtf(D) - R")


def _rotations(rng, n):
    qv = rng.normal(size=(n, 4))
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    w, x, y, z = qv.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def test_ray_setup_matches_the_reference_expression(probe):
    lib, torch = probe
    rng = np.random.default_rng(3)
    n = 2_000_000
    R = _rotations(rng, n)
    M = np.zeros((n, 4, 4))
    M[:, :3, :3] = R
    M[:, :3, 3] = rng.uniform(-1, 9, (n, 3))
    M[: n // 8, :3, 3] += 1e4
    M[:, 3, 3] = 1.0
    m_colmajor = np.ascontiguousarray(np.transpose(M, (0, 2, 1)).reshape(n, 16)).astype(np.float32)
    W = rng.integers(16, 4097, n).astype(np.int32)
    H = rng.integers(16, 2161, n).astype(np.int32)
    fov = rng.uniform(0.3, 2.5, n)
    pane = (W / (2 * np.tan(0.5 * fov))).astype(np.float32)
    x = (rng.random(n) * W).astype(np.int32)
    y = (rng.random(n) * H).astype(np.int32)
    md = _dev(torch, m_colmajor)
    whd = _dev(torch, np.stack([W, H], 1).astype(np.int32))
    pd = _dev(torch, pane)
    xyd = _dev(torch, np.stack([x, y], 1).astype(np.int32))
    ref = torch.empty((n, 5), dtype=torch.float32, device="cuda")
    got = torch.empty_like(ref)
    assert lib.fpc_ray(md.data_ptr(), whd.data_ptr(), pd.data_ptr(), xyd.data_ptr(), n, ref.data_ptr(),
                       got.data_ptr()) == 0
    _same_bits(ref, got, "ray direction, t_near, t_far")
