"""bhut/tree/node.py: the ``TreeData`` container of a built tree.

The same fields as the reference's (node id order, children of internal
node k at first_child[k] .. first_child[k] + child_count[k] - 1, particles of
node k at perm[start[k] : start[k] + count[k]]); ``Tree._tree`` and the
module-level stages of ``bhut_gb300.tree`` and ``bhut_gb300.traverse``
return or accept it.  Here it is a host copy of the device tree
(``bhut_tree_export``), and ``bhut_tree_import`` loads one back.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class TreeData:
    """Host copy of the device tree with the reference's TreeData fields."""

    center: np.ndarray
    half_size: np.ndarray
    mass: np.ndarray
    com: np.ndarray
    first_child: np.ndarray
    child_count: np.ndarray
    start: np.ndarray
    count: np.ndarray
    is_leaf: np.ndarray
    perm: np.ndarray
    dim: int
    leaf_size: int

    @property
    def num_nodes(self) -> int:
        return len(self.center)

    @property
    def num_particles(self) -> int:
        return len(self.perm)

    def validate(self) -> None:
        """Consistency checks of bhut/tree/node.py:83-134 (shapes, root count,
        permutation, child indices, leaf sizes), same messages."""
        M, N, D = self.num_nodes, self.num_particles, self.dim
        if D not in (2, 3):
            raise ValueError(f"dim must be 2 or 3, got {D}")
        for name, arr, want in (("center", self.center, (M, D)), ("half_size", self.half_size, (M,)),
                                ("mass", self.mass, (M,)), ("com", self.com, (M, D)),
                                ("first_child", self.first_child, (M,)),
                                ("child_count", self.child_count, (M,)),
                                ("start", self.start, (M,)), ("count", self.count, (M,)),
                                ("is_leaf", self.is_leaf, (M,))):
            if np.shape(arr) != want:
                raise ValueError(f"{name} has shape {np.shape(arr)}, expected {want}")
        if np.shape(self.perm) != (N,):
            raise ValueError(f"perm has shape {np.shape(self.perm)}, expected ({N},)")
        if M > 0:
            if self.count[0] != N:
                raise ValueError(f"Root node count {self.count[0]} != num_particles {N}")
            if not np.array_equal(np.sort(self.perm), np.arange(N)):
                raise ValueError("perm is not a valid permutation")
            fc = np.asarray(self.first_child)
            if np.any(fc[fc >= 0] >= M):
                raise ValueError("first_child indices exceed number of nodes")
            if np.any(np.asarray(self.count)[np.asarray(self.is_leaf)] > self.leaf_size):
                raise ValueError("Some leaf nodes exceed leaf_size")

    def get_children(self, node_idx: int) -> np.ndarray:
        if self.is_leaf[node_idx]:
            return np.array([], dtype=np.intp)
        first = self.first_child[node_idx]
        return np.arange(first, first + self.child_count[node_idx], dtype=np.intp)

    def get_particles(self, node_idx: int) -> np.ndarray:
        s = self.start[node_idx]
        return self.perm[np.arange(s, s + self.count[node_idx], dtype=np.intp)]
