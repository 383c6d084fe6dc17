"""In-tree build of the CUDA library (``lib/librm_gb300.so``) and the
``marcher.bin`` command-line driver.

nvcc compiles each translation unit for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``) in parallel, then links one shared
library with a plain C ABI (``include/rm.h``).  Nothing is installed
outside the repository.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "librm_gb300.so")
CLI = os.path.join(LIBDIR, "marcher.bin")
IOLIB = os.path.join(LIBDIR, "librm_io.so")

CUDA_SOURCES = ["rm_index.cu", "rm_radii.cu", "rm_march.cu", "rm_backward.cu", "rm_api.cu",
                "rm_noalloc.cu"]
HOST_SOURCES = ["marcher_main.cpp", "io.cpp", "rmio_c.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _digest(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def _headers():
    out = [os.path.join(INCLUDE, "rm.h"), os.path.join(INCLUDE, "rmio.h")]
    for d in (CSRC, HOST):
        if os.path.isdir(d):
            out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh", ".hpp"))]
    return out


def _compile(src: str, obj: str, flags) -> None:
    cmd = [_nvcc()] + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-4000:]))


def build_host() -> None:
    """librm_io.so (file formats, no CUDA) and marcher.bin (links both libraries)."""
    io_srcs = [os.path.join(HOST, "io.cpp"), os.path.join(HOST, "rmio_c.cpp")]
    tmp = IOLIB + ".tmp%d" % os.getpid()
    cmd = (["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-I" + INCLUDE,
            "-I" + HOST, "-o", tmp] + io_srcs + ["-lz"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("io library build failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, IOLIB)
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = (["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + INCLUDE, "-I" + HOST, "-o", tmp,
            os.path.join(HOST, "marcher_main.cpp"), "-L" + LIBDIR, "-lrm_io", "-lrm_gb300",
            "-Wl,-rpath,$ORIGIN", "-lz", "-lm", "-lpthread"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, CLI)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library (and the CLI when its sources exist); return the
    path of the shared library."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES]
    hsrcs = [os.path.join(HOST, s) for s in HOST_SOURCES if os.path.exists(os.path.join(HOST, s))]
    stamp = os.path.join(OBJDIR, "stamp")
    digest = _digest(srcs + hsrcs + _headers(), " ".join(NVCC_FLAGS) + os.uname().machine)
    if (not force and os.path.exists(LIB) and os.path.exists(stamp)
            and open(stamp).read().strip() == digest
            and (not hsrcs or (os.path.exists(CLI) and os.path.exists(IOLIB)))):
        return LIB
    objs = [os.path.join(OBJDIR, os.path.basename(s) + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, NVCC_FLAGS) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIB)
    if hsrcs:
        build_host()
    with open(stamp, "w") as f:
        f.write(digest)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
