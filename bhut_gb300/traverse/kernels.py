"""bhut/traverse/kernels.py:171-197 ``validate_kernel_inputs`` (host checks,
same messages).  The pair and monopole arithmetic itself lives in the CUDA
traversal kernels."""
from __future__ import annotations

import numpy as np

from ..api import _host, _is_torch, _shape


def validate_kernel_inputs(positions, masses, softening) -> None:
    """Shape checks of the traversal inputs (softening checked against the
    sources)."""
    ps, ms = _shape(positions), _shape(masses)
    if len(ps) != 2:
        raise ValueError(f"positions must be 2D array, got shape {ps}")
    if len(ms) != 1:
        raise ValueError(f"masses must be 1D array, got shape {ms}")
    if ps[0] != ms[0]:
        raise ValueError(f"positions has {ps[0]} particles but masses has {ms[0]} elements")
    if not np.isscalar(softening):
        s = np.asarray(_host(softening) if _is_torch(softening) else softening)
        if len(s.shape) != 1:
            raise ValueError(f"softening must be scalar or 1D array, got shape {s.shape}")
        if s.shape[0] != ps[0]:
            raise ValueError(f"softening array has {s.shape[0]} elements but need {ps[0]}")
