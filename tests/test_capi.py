"""The C-ABI library loads and exports every entry point of include/*.h
(no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import REPO


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"BHUT_API\s+[\w\s\*]*?\b(bhut_\w+)\s*\(", text))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("bhut_tree_create", "bhut_tree_build", "bhut_tree_refit",
                     "bhut_tree_rebuild", "bhut_tree_accel_self", "bhut_tree_accel_targets",
                     "bhut_tree_export", "bhut_tree_destroy", "bhut_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(engine_lib):
    from bhut_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    # the Python binding covers exactly the declared symbols
    assert set(_lib.SIGNATURES) == declared_symbols()


def test_version_and_error_buffer(engine_lib):
    from bhut_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.bhut_version()
    buf = ctypes.create_string_buffer(8)
    n = L.bhut_last_error(buf, len(buf))
    assert n >= 0


def test_invalid_arguments_rejected_before_device_work(engine_lib):
    """Argument checks that need no GPU return BHUT_EINVAL with the reference's
    message."""
    from bhut_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.bhut_tree_create(4, 32, None, ctypes.byref(h)) == _lib.BHUT_EINVAL
    assert "dim must be 2 or 3" in _lib.last_error()
    assert L.bhut_tree_create(3, 0, None, ctypes.byref(h)) == _lib.BHUT_EINVAL
    assert "leaf_size must be positive" in _lib.last_error()
    assert L.bhut_morton_keys(None, 0, 3, None, None) == _lib.BHUT_EINVAL


def test_more_invalid_arguments(engine_lib):
    """Argument checks of the newer entry points, before any device work."""
    from bhut_gb300 import _lib
    L = _lib.load()
    E = _lib.BHUT_EINVAL
    assert L.bhut_batch_configure(None, 2, 0, 32, 1) == E
    assert L.bhut_batch_set_multipole(None, 1) == E
    assert L.bhut_batch_set_stack(None, 1) == E
    assert L.bhut_tree_set_multipole(None, 0) == E
    assert L.bhut_tree_set_criterion(None, 0) == E
    assert L.bhut_morton_codes_unit(None, 10, 4, 21, None, None) == E
    assert "points01 must have 2 or 3 dimensions" in _lib.last_error()
    assert L.bhut_morton_codes_unit(None, 10, 3, 0, None, None) == E
    assert "bits must be in 1..62" in _lib.last_error()
    assert L.bhut_sort_morton_unit(None, 10, 3, 63, None, None, None) == E
    assert L.bhut_gather_rows(None, -1, 8, None, None, None) == E
    assert L.bhut_should_refit(None, 10, 4, None, 1.0, None, None) == E
    assert L.bhut_tree_statistics(None, None, None, None, None, None, None, 0, 3, None, 0, 0.5,
                                  None, None) == E
    assert L.bhut_tree_import(None, None, None, 0, None, None, None, None, None, None, None,
                              None, None, 0) == E
    assert L.bhut_tree_refit_only(None, None, None, 0) == E
    assert L.bhut_measure_fp32_peak(None) == E
    assert L.bhut_aabb(None, 0, 3, None, None, None) == E
    assert "points array cannot be empty" in _lib.last_error()
