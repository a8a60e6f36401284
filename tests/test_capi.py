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
    # calls on no context are refused before any device work
    fields = (ctypes.c_int32 * 2)(0, 64)
    assert lib.g5_pack_fields(None, None, fields, 2, 0, 1, None, None) == -1
    assert lib.g5_derived_quantity(None, None, 0, 0, 1, None, None) == -1
    assert lib.g5_set_shape(None, 0, (ctypes.c_int32 * 4)(0, 1, 1, 0)) == -1


def test_tune_pick_selection_rule():
    """g5_tune's selection (host only): the fastest candidate, but the default
    shape stays while it is within the margin of the fastest."""
    from godunov_five_eq_gb300.implem import G5Error, tune_pick, unpack_shape

    assert tune_pick([3.0, 2.0, 2.5], default_index=0) == 1
    assert tune_pick([2.03, 2.0, 2.5], default_index=0, margin=0.02) == 0  # within 2 %
    assert tune_pick([2.05, 2.0, 2.5], default_index=0, margin=0.02) == 1
    assert tune_pick([0.0, 2.0, 1.0], default_index=1) == 2  # a failed (zero) timing never wins
    assert tune_pick([5.0], default_index=0) == 0
    with pytest.raises(G5Error):
        tune_pick([1.0, 2.0], default_index=2)
    with pytest.raises(G5Error):
        tune_pick([0.0, 0.0], default_index=0)
    assert unpack_shape(4 + 16 + 32) == {"ctas_per_sm": 4, "claim": 1, "walk_cf_first": 1, "reflux_layout": 0}
    assert unpack_shape(2 + 64) == {"ctas_per_sm": 2, "claim": 0, "walk_cf_first": 0, "reflux_layout": 1}
    assert unpack_shape(3 + 16 + 128) == {"ctas_per_sm": 3, "claim": 1, "walk_cf_first": 0, "reflux_layout": 2}
