"""bhut/traverse/bh.py on the GPU: ``barnes_hut_accelerations`` (:428-482),
``barnes_hut_accelerations_targets`` (:30-80) and ``compute_tree_statistics``
(:604-700), same signatures.  The given TreeData is loaded onto the device
as it is (refitted trees included) and traversed by the engine's kernels;
``form`` selects the arithmetic as in ``bhut_gb300.accelerations``."""
from __future__ import annotations

from ..api import (DEFAULT_FORM, _empty_like_out, _Handle, _scalar_softening, _shape, _to_f64,
                   compute_tree_statistics)  # noqa: F401
from .kernels import validate_kernel_inputs


def _loaded(tree, positions, masses, form):
    h = _Handle(tree.dim, tree.leaf_size)
    h.set_form(form or DEFAULT_FORM)
    h.import_tree(tree, positions, masses)
    return h


def barnes_hut_accelerations(tree, positions, masses, softening, theta: float = 0.5,
                             G: float = 1.0, *, form: str | None = None):
    """Self accelerations of the particles the tree was built on."""
    positions = _to_f64(positions)
    masses = _to_f64(masses)
    validate_kernel_inputs(positions, masses, softening)
    n = _shape(positions)[0]
    eps = _scalar_softening(softening, n)
    out = _empty_like_out(positions, (n, _shape(positions)[1]))
    h = _loaded(tree, positions, masses, form)
    try:
        h.accel_self(theta, eps, G, out)
    finally:
        h.close()
    return out


def barnes_hut_accelerations_targets(tree, tree_positions, tree_masses, target_positions,
                                     softening, theta: float = 0.5, G: float = 1.0, *,
                                     form: str | None = None):
    """Accelerations at arbitrary targets due to the tree's particles."""
    tree_positions = _to_f64(tree_positions)
    tree_masses = _to_f64(tree_masses)
    target_positions = _to_f64(target_positions)
    validate_kernel_inputs(tree_positions, tree_masses, softening)
    eps = _scalar_softening(softening, _shape(tree_positions)[0])
    m = _shape(target_positions)[0]
    out = _empty_like_out(target_positions, (m, _shape(target_positions)[1]))
    if m == 0:
        return out
    h = _loaded(tree, tree_positions, tree_masses, form)
    try:
        h.accel_targets(target_positions, theta, eps, G, out)
    finally:
        h.close()
    return out
