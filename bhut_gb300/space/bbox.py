"""bhut/space/bbox.py on the GPU: ``aabb`` (:14-46) and ``normalize_to_unit``
(:49-96), same signatures, checks and messages; NumPy in → NumPy out, CUDA
tensors in → CUDA tensors out."""
from __future__ import annotations

import numpy as np

from .. import _lib
from ..api import _empty_like_out, _is_cuda_tensor, _ptr, _shape, _sync_torch, _to_f64, _torch


def _out_vec(ref, values: np.ndarray):
    if _is_cuda_tensor(ref):
        return _torch().as_tensor(values, device=ref.device)
    return values


def aabb(points):
    """Per-axis (min, max) of the points (N, D)."""
    points = _to_f64(points)
    shape = _shape(points)
    if len(shape) != 2:
        raise ValueError(f"points must be 2D array, got shape {shape}")
    if shape[0] == 0:
        raise ValueError("points array cannot be empty")
    d = shape[1]
    if not 1 <= d <= 3:
        raise ValueError(f"points must have 1 to 3 dimensions, got {d}")
    pmin = np.empty(d)
    pmax = np.empty(d)
    _sync_torch(points)
    _lib.check(_lib.load().bhut_aabb(_ptr(points), shape[0], d, pmin.ctypes.data,
                                     pmax.ctypes.data, None))
    return _out_vec(points, pmin), _out_vec(points, pmax)


def normalize_to_unit(points, pmin, pmax, eps: float = 1e-12):
    """(points - pmin) / extent + offset, degenerate axes at 0.5, clamped at
    1 - eps."""
    points = _to_f64(points)
    shape = _shape(points)
    lo = np.ascontiguousarray(np.asarray(_host_vec(pmin), dtype=np.float64).reshape(-1))
    hi = np.ascontiguousarray(np.asarray(_host_vec(pmax), dtype=np.float64).reshape(-1))
    d = shape[1] if len(shape) == 2 else 0
    if len(shape) != 2 or not 1 <= d <= 3 or lo.shape != (d,) or hi.shape != (d,):
        raise ValueError(f"points {shape} and bounds {lo.shape}, {hi.shape} do not match")
    out = _empty_like_out(points, shape)
    _sync_torch(points, out)
    _lib.check(_lib.load().bhut_normalize_to_unit(_ptr(points), shape[0], d, lo.ctypes.data,
                                                  hi.ctypes.data, float(eps), _ptr(out), None))
    return out


def _host_vec(v):
    if hasattr(v, "detach") and hasattr(v, "cpu"):
        return v.detach().cpu().numpy()
    return v
