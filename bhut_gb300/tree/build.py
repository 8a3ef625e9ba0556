"""bhut/tree/build.py:19-107 ``build_tree`` on the GPU: bounding box, Morton
keys, stable radix sort, count-split topology and bottom-up node moments in
the engine's kernels; the TreeData it returns is bit-identical to the
reference's."""
from __future__ import annotations

from ..api import _Handle, _shape, _to_f64


def build_tree(positions, masses, *, dim: int, leaf_size: int, xp=None, multipole: str = "mono"):
    """Same signature as the reference; ``xp`` is accepted and unused (the
    arrays are NumPy or torch)."""
    if multipole != "mono":
        raise ValueError(f"multipole must be 'mono', got '{multipole}'")
    positions = _to_f64(positions)
    masses = _to_f64(masses)
    if _shape(positions)[0] == 0:
        raise ValueError("Cannot build tree with zero particles")
    h = _Handle(dim, leaf_size)
    try:
        h.build(positions, masses)
        return h.export()
    finally:
        h.close()
