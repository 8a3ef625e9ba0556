"""ctypes binding of libbhut_gb300.so (the C ABI in include/bhut_gb300.h).

The library must have been built (``python -m bhut_gb300._build`` or
``__graft_entry__.build()``); importing the engine without it fails loudly --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libbhut_gb300.so")

BHUT_OK = 0
BHUT_EINVAL = 1
BHUT_ENOTBUILT = 2
BHUT_ECUDA = 3
BHUT_ENOMEM = 4
BHUT_EDEVICE = 5
BHUT_EINTERNAL = 6

FORM_EXACT = 0
FORM_FAST = 1
FORM_FP32 = 2
FORMS = {"exact": FORM_EXACT, "fast": FORM_FAST, "fp32": FORM_FP32}
MAC_BH = 0
MAC_OFFSET = 1
CRITERIA = {"bh": MAC_BH, "bh_offset": MAC_OFFSET}
MULTIPOLES = {"mono": 0, "quad": 1}
STACKS = {"shared": 0, "registers": 1}

_VP = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int

# name -> (restype, argtypes); every symbol here is declared in the header
SIGNATURES = {
    "bhut_version": (ctypes.c_char_p, []),
    "bhut_last_error": (_INT, [ctypes.c_char_p, ctypes.c_size_t]),
    "bhut_tree_create": (_INT, [_INT, _INT, _VP, ctypes.POINTER(_VP)]),
    "bhut_tree_build": (_INT, [_VP, _VP, _VP, _I64]),
    "bhut_tree_refit": (_INT, [_VP, _VP, _VP, _I64, ctypes.POINTER(_INT)]),
    "bhut_tree_rebuild": (_INT, [_VP, _VP, _VP, _I64]),
    "bhut_tree_accel_self": (_INT, [_VP, _D, _D, _D, _VP]),
    "bhut_tree_accel_targets": (_INT, [_VP, _VP, _I64, _D, _D, _D, _VP]),
    "bhut_tree_set_form": (_INT, [_VP, _INT]),
    "bhut_tree_set_criterion": (_INT, [_VP, _INT]),
    "bhut_tree_set_multipole": (_INT, [_VP, _INT]),
    "bhut_tree_info": (_INT, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                              ctypes.POINTER(_INT), ctypes.POINTER(_INT)]),
    "bhut_tree_export": (_INT, [_VP] * 11),
    "bhut_tree_destroy": (None, [_VP]),
    "bhut_tree_stats": (_INT, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                               ctypes.POINTER(_I64)]),
    "bhut_tree_fallbacks": (_INT, [_VP, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "bhut_launch_count": (ctypes.c_longlong, []),
    "bhut_morton_keys": (_INT, [_VP, _I64, _INT, _VP, _VP]),
    "bhut_morton_argsort": (_INT, [_VP, _I64, _INT, _VP, _VP, _VP]),
    "bhut_direct_accelerations": (_INT, [_VP, _VP, _I64, _INT, _VP, _I64, _D, _D, _VP, _VP]),
    "bhut_tree_statistics": (_INT, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _I64, _INT, _VP, _I64, _D,
                                    _VP, _VP]),
    "bhut_aabb": (_INT, [_VP, _I64, _INT, _VP, _VP, _VP]),
    "bhut_normalize_to_unit": (_INT, [_VP, _I64, _INT, _VP, _VP, _D, _VP, _VP]),
    "bhut_morton_codes_unit": (_INT, [_VP, _I64, _INT, _INT, _VP, _VP]),
    "bhut_sort_morton_unit": (_INT, [_VP, _I64, _INT, _INT, _VP, _VP, _VP]),
    "bhut_gather_rows": (_INT, [_VP, _I64, _I64, _VP, _VP, _VP]),
    "bhut_should_refit": (_INT, [_VP, _I64, _INT, _VP, _D, _VP, _VP]),
    "bhut_tree_refit_only": (_INT, [_VP, _VP, _VP, _I64]),
    "bhut_measure_fp32_peak": (_INT, [_VP]),
    "bhut_pool_usage": (_INT, [_VP, _VP]),
    "bhut_pool_trim": (_INT, []),
    "bhut_tree_import": (_INT, [_VP, _VP, _VP, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                _I64]),
    "bhut_morton_argsort_noalloc": (_INT, [_VP, _I64, _INT, _VP, _VP, _VP]),
    "bhut_batch_create": (_INT, [_INT, _INT, _VP, ctypes.POINTER(_VP)]),
    "bhut_batch_configure": (_INT, [_VP, _INT, _INT, _INT, _INT]),
    "bhut_batch_set_multipole": (_INT, [_VP, _INT]),
    "bhut_batch_set_stack": (_INT, [_VP, _INT]),
    "bhut_batch_roots": (_INT, [_VP, _VP]),
    "bhut_batch_set_refit_rule": (_INT, [_VP, _INT]),
    "bhut_batch_set_roots": (_INT, [_VP, _VP]),
    "bhut_batch_forced": (_INT, [_VP, _VP]),
    "bhut_batch_outside": (_INT, [_VP, _VP, _VP]),
    "bhut_batch_load": (_INT, [_VP, _VP, _VP, _VP, _I64]),
    "bhut_batch_solve": (_INT, [_VP, _D, _D, _D, _VP]),
    "bhut_batch_info": (_INT, [_VP] + [ctypes.POINTER(_I64)] * 4),
    "bhut_batch_stats": (_INT, [_VP] + [ctypes.POINTER(_I64)] * 3),
    "bhut_batch_keep_order": (_INT, [_VP, _VP, _VP]),
    "bhut_batch_order": (_INT, [_VP, _VP]),
    "bhut_batch_destroy": (None, [_VP]),
    "bhut_batch_traverse_ms": (_INT, [_VP, _VP]),
    "bhut_leapfrog": (_INT, [_VP, _VP, _VP, _I64, _INT, _D, _D, _VP]),
}

_lock = threading.Lock()
_lib = None


class EngineError(RuntimeError):
    """A CUDA-side failure reported by the engine."""


def load():
    """Load the shared library and bind every C-ABI entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA engine first "
                "(python -m bhut_gb300._build, or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def last_error() -> str:
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.bhut_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    """Map a C-ABI status to the exception type the reference raises."""
    if status == BHUT_OK:
        return
    msg = last_error()
    if status in (BHUT_EINVAL, BHUT_ENOTBUILT):
        raise ValueError(msg)
    if status == BHUT_ENOMEM:
        raise MemoryError(msg)
    raise EngineError(msg)
