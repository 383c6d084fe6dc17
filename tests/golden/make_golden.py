"""Generate the golden vectors under tests/golden/ from the reference's own
FLANN CPU kd-tree (oracle/_ref/ref_driver, built by oracle/Makefile.ref from
the reference tree).  Run where the reference is present:

    make -f oracle/Makefile.ref REF=<reference checkout>
    python tests/golden/make_golden.py

Fixtures (numpy .npz, seeded synthetic inputs):
  knn_flann.npz    the cloud (xyz) + queries, FLANN's raw 10-NN and 2-NN answers
  radii_flann.npz  the reference radii rule evaluated on FLANN's neighbours
The cloud is stored once, in knn_flann.npz.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from renderer_ray_marching_gb300 import synthetic as syn  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def run(*args):
    subprocess.run([DRIVER] + [str(a) for a in args], check=True)


def cloud(n: int, seed: int):
    sc = syn.make_scene(n, n_boxes=12, seed=seed)
    xyz = sc.xyz.copy()
    # exact duplicates and an isolated far point: tie and far-query cases
    xyz[10:14] = xyz[3]
    xyz[-1] = np.array([40.0, -7.0, 12.0], np.float32)
    return xyz, sc


def main():
    if not os.path.exists(DRIVER):
        raise SystemExit("build oracle/_ref/ref_driver first (make -f oracle/Makefile.ref)")
    rng = np.random.default_rng(7)
    xyz, sc = cloud(30000, seed=11)
    n = xyz.shape[0]
    q_pts = xyz[rng.choice(n, 1000, replace=False)]
    q_room = rng.uniform([-0.5, -0.5, -0.5], [8.5, 6.5, 3.5], size=(1500, 3)).astype(np.float32)
    q_far = rng.uniform(-60, 60, size=(100, 3)).astype(np.float32)
    queries = np.concatenate([q_pts, q_room, q_far]).astype(np.float32)
    m = queries.shape[0]
    with tempfile.TemporaryDirectory() as td:
        P = os.path.join(td, "p.f32"); xyz.tofile(P)
        Q = os.path.join(td, "q.f32"); queries.tofile(Q)
        out = {}
        for k in (2, 10):
            I = os.path.join(td, "i.i32"); D = os.path.join(td, "d.f32")
            run("knn", P, n, Q, m, k, I, D)
            out["idx%d" % k] = np.fromfile(I, np.int32).reshape(m, k)
            out["d2_%d" % k] = np.fromfile(D, np.float32).reshape(m, k)
        np.savez_compressed(os.path.join(HERE, "knn_flann.npz"), xyz=xyz, queries=queries, **out)

        R = os.path.join(td, "r.f32"); NN = os.path.join(td, "nn.i32")
        run("radii", P, n, R, NN)
        radii = np.fromfile(R, np.float32)
        nn = np.fromfile(NN, np.int32)
        np.savez_compressed(os.path.join(HERE, "radii_flann.npz"), radii=radii, nn=nn)

    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
