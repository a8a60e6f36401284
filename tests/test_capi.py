"""The C-ABI library builds for sm_103a, loads, and exports every symbol
include/g5gpu.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

from godunov_five_eq_gb300 import implem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "g5gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(g5_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_declared_symbols():
    lib = implem.load_library()
    syms = declared_symbols()
    assert "g5_step" in syms and "g5_set_mesh" in syms
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(implem.EXPORTS)
    assert lib.g5_version().startswith(b"g5gpu")


def test_invalid_params_rejected_without_device():
    lib = implem.load_library()
    p = implem.G5Params()
    p.dim = 5
    ctx = ctypes.c_void_p()
    assert lib.g5_create(ctypes.byref(p), ctypes.byref(ctx)) == -1
    p.dim = 2
    p.bsize = 7
    assert lib.g5_create(ctypes.byref(p), ctypes.byref(ctx)) == -1
    assert lib.g5_create(None, ctypes.byref(ctx)) == -1
    assert lib.g5_destroy(None) == -1
