"""bhut/tree/refit.py on the GPU: ``refit_tree`` (:17-109) and
``should_refit_vs_rebuild`` (:195-251), same signatures, checks and
messages."""
from __future__ import annotations

import numpy as np

from .. import _lib
from ..api import _Handle, _ptr, _shape, _sync_torch, _to_f64


def refit_tree(tree, new_positions, masses, xp=None):
    """A new TreeData with masses and centres of mass recomputed for
    ``new_positions`` (original order) through the tree's frozen permutation;
    geometry and topology are kept."""
    new_positions = _to_f64(new_positions)
    masses = _to_f64(masses)
    n = len(tree.perm)
    if _shape(new_positions)[0] != n:
        raise ValueError(f"new_positions has {_shape(new_positions)[0]} particles "
                         f"but tree was built with {n} particles")
    if _shape(masses)[0] != n:
        raise ValueError(f"masses has {_shape(masses)[0]} elements "
                         f"but tree was built with {n} particles")
    if _shape(new_positions)[1] != tree.dim:
        raise ValueError(f"new_positions has {_shape(new_positions)[1]} dimensions "
                         f"but tree has {tree.dim} dimensions")
    h = _Handle(tree.dim, tree.leaf_size)
    try:
        h.import_tree(tree, new_positions, masses)
        h.refit_only(new_positions, masses)
        return h.export()
    finally:
        h.close()


def should_refit_vs_rebuild(tree, new_positions, position_tolerance: float = 0.1,
                            boundary_check: bool = True) -> bool:
    """True (refit) unless the particle count or dimension changed or, with
    ``boundary_check``, a particle lies beyond 1.1 x the root half-size from
    the root centre along some axis."""
    new_positions = _to_f64(new_positions)
    shape = _shape(new_positions)
    if shape[0] != len(tree.perm):
        return False
    if shape[1] != tree.dim:
        return False
    if boundary_check:
        center = np.ascontiguousarray(np.asarray(tree.center)[0], dtype=np.float64)
        res = np.zeros(1, dtype=np.int32)
        _sync_torch(new_positions)
        _lib.check(_lib.load().bhut_should_refit(_ptr(new_positions), shape[0], shape[1],
                                                 center.ctypes.data,
                                                 float(np.asarray(tree.half_size)[0]),
                                                 res.ctypes.data, None))
        return bool(res[0])
    return True
