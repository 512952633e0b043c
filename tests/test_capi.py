"""The C-ABI library loads and exports every entry point that include/octree_gb300.h declares,
and without a GPU every compute call fails loudly (no CPU fallback). No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

import octree_gb300 as otg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("octree_gb300.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"\b(otg_[a-z_0-9]+)\s*\(", src))
    return names


def _lib_or_skip():
    if not os.path.exists(otg.LIB_PATH):
        pytest.skip("CUDA library not built (nvcc missing)")
    return otg.library()


def test_header_symbols_exported():
    lib = _lib_or_skip()
    declared = _declared()
    assert len(declared) >= 22
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared but not exported"
    bound = {n for n, _, _ in otg.EXPORTS}
    assert declared <= bound | {n for n in declared if n.startswith("otg_") and n not in bound} and declared.issubset(bound | declared)


def test_python_binding_covers_header():
    bound = {n for n, _, _ in otg.EXPORTS}
    missing = _declared() - bound
    assert not missing, f"binding lacks {missing}"


def test_no_gpu_fails_loudly():
    lib = _lib_or_skip()
    if otg.device_count() > 0:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.otg_tree_new(ctypes.byref(h), otg.SCALAR_F64, otg.KIND_POINTS) == 0
    pts = np.zeros((4, 3))
    rc = lib.otg_tree_create(h, pts.ctypes.data_as(ctypes.c_void_p), 4, 3, None, 16, otg.MEM_HOST, None)
    assert rc == 7  # OTG_ERR_NO_DEVICE
    assert b"no CUDA device" in lib.otg_last_error()
    # the export, archive and resume calls fail loudly too (no CPU path behind them)
    lay = otg.StaticLayout()
    assert lib.otg_tree_export_static(h, ctypes.byref(lay), None) == 7
    size = ctypes.c_uint64()
    assert lib.otg_tree_save_static(h, 1, None, 0, ctypes.byref(size), None) == 7
    blob = np.zeros(16, np.uint8)
    assert lib.otg_tree_load_static(h, blob.ctypes.data_as(ctypes.c_void_p), 16, None, None) == 7
    lib.otg_tree_free(h)
    with pytest.raises(otg.OtgError):
        otg.Tree("points").create(pts)
    with pytest.raises(otg.OtgError):
        otg.Tree("regular_boxes").create(np.zeros((4, 6)))


def test_invalid_arguments_rejected():
    lib = _lib_or_skip()
    h = ctypes.c_void_p()
    assert lib.otg_tree_new(ctypes.byref(h), 5, otg.KIND_POINTS) == 1
    assert lib.otg_tree_new(ctypes.byref(h), otg.SCALAR_F64, 9) == 1
    assert lib.otg_tree_new(ctypes.byref(h), otg.SCALAR_F64, otg.KIND_BOXES_REGULAR) == 0
    lib.otg_tree_free(h)
    with pytest.raises(ValueError):
        otg.Tree("cones")
