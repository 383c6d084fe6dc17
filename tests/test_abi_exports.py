"""The C-ABI library loads and exports every symbol that include/rm.h
declares (no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import numpy as np

from renderer_ray_marching_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "rm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rm_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_header_symbols():
    lib = ctypes.CDLL(build.build())
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(_abi.EXPORTS) == syms


def test_config_default_is_reference_constants():
    lib = _abi.load()
    cfg = _abi.RmConfig()
    lib.rm_config_default(ctypes.byref(cfg))
    f32 = lambda x: float(np.float32(x))
    assert cfg.zfar == 100.0 and cfg.znear == f32(0.1) and cfg.max_steps == 128
    assert cfg.min_dist == f32(0.001) and cfg.knn == 10 and cfg.leaf_size == 16


def test_null_context_is_rejected_not_crashing():
    lib = _abi.load()
    assert lib.rm_synchronize(None) == _abi.RM_ERR_INVALID
    assert lib.rm_last_error(None) == b"null context"
    assert lib.rm_cloud_size(None) == -1


def test_python_constants_and_structs_mirror_the_header():
    text = open(os.path.join(ROOT, "include", "rm.h")).read()
    assert int(re.search(r"#define RM_NOALLOC_MAX_VIEWS (\d+)", text).group(1)) == _abi.RM_NOALLOC_MAX_VIEWS
    end = text.index("} rm_stats;")
    body = text[text.rindex("typedef struct {", 0, end):end]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\b(?:int64_t|float)\s+([a-z_]+)\s*;", body)
    assert fields == [f for f, _ in _abi.RmStats._fields_]
