"""bhut/utils/morton.py on the GPU: ``morton_codes`` (:48-102) and
``sort_by_morton`` (:105-147), same signatures, checks and messages.  The
codes come from the same quantisation and bit interleave as the reference
(bit-exact); the sort is the engine's stable LSD radix sort."""
from __future__ import annotations

import numpy as np

from .. import _lib
from ..api import _is_cuda_tensor, _ptr, _shape, _sync_torch, _to_f64, _torch


def _check_points01(points01):
    points01 = _to_f64(points01)
    shape = _shape(points01)
    if len(shape) != 2:
        raise ValueError(f"points01 must be 2D array, got shape {shape}")
    if shape[1] not in (2, 3):
        raise ValueError(f"points01 must have 2 or 3 dimensions, got {shape[1]}")
    return points01, shape


def _empty(ref, n, dtype_np, dtype_torch):
    if _is_cuda_tensor(ref):
        return _torch().empty(n, dtype=dtype_torch, device=ref.device)
    return np.empty(n, dtype=dtype_np)


def morton_codes(points01, bits: int = 21):
    """Morton codes (uint64) of points in [0, 1)^D, D = 2 or 3."""
    points01, (n, d) = _check_points01(points01)
    codes = _empty(points01, n, np.uint64, _torch().uint64 if _is_cuda_tensor(points01) else None)
    if n:
        _sync_torch(points01, codes)
        _lib.check(_lib.load().bhut_morton_codes_unit(_ptr(points01), n, d, int(bits),
                                                      _ptr(codes), None))
    return codes


def sort_by_morton(points01, data_arrays=None, bits: int = 21):
    """(codes in sorted order, perm, [data arrays permuted to sorted order])."""
    points01, (n, d) = _check_points01(points01)
    cuda = _is_cuda_tensor(points01)
    codes = _empty(points01, n, np.uint64, _torch().uint64 if cuda else None)
    perm = _empty(points01, n, np.intp, _torch().int64 if cuda else None)
    if n:
        _sync_torch(points01, codes, perm)
        _lib.check(_lib.load().bhut_sort_morton_unit(_ptr(points01), n, d, int(bits),
                                                     _ptr(codes), _ptr(perm), None))
    sorted_data = []
    if data_arrays is not None:
        for arr in data_arrays:
            if not (hasattr(arr, "data_ptr") and hasattr(arr, "is_cuda")):
                arr = np.asarray(arr)
            if arr.shape[0] != n:
                raise ValueError(f"Data array has {arr.shape[0]} elements but need {n}")
            sorted_data.append(_gather(arr, perm))
    return codes, perm, sorted_data


def _gather(arr, perm):
    """arr[perm] along the first axis, on the GPU."""
    n = arr.shape[0]
    if hasattr(arr, "data_ptr"):                      # torch tensor
        src = arr.contiguous()
        out = _torch().empty_like(src)
        row = src.element_size() * (src.numel() // max(n, 1))
        p = perm if hasattr(perm, "data_ptr") else _torch().as_tensor(perm)
        if src.is_cuda:
            p = p.to(src.device)
        _sync_torch(src, out, p)
    else:
        src = np.ascontiguousarray(arr)
        out = np.empty_like(src)
        row = src.itemsize * (src.size // max(n, 1))
        p = perm.cpu().numpy() if hasattr(perm, "cpu") else np.ascontiguousarray(perm,
                                                                                  dtype=np.int64)
    if n and row:
        _lib.check(_lib.load().bhut_gather_rows(_ptr(src), n, row, _ptr(p), _ptr(out), None))
    return out
