"""CPU oracle for the Barnes-Hut hot path -- TEST INFRASTRUCTURE ONLY.

This module wraps ``bhut_oracle.c`` (a scalar FP64 restatement of bhut 0.1.0:
``bhut/space/bbox.py``, ``bhut/utils/morton.py``, ``bhut/tree/build.py``,
``bhut/tree/refit.py``, ``bhut/traverse/bh.py`` and
``bhut/traverse/kernels.py``) for the test suite, the smoke check and the
CPU-baseline leg of ``bench.py``.  The CUDA engine in ``bhut_gb300`` never
imports it.

Parity of this oracle with the reference is pinned by the golden fixtures in
``tests/golden`` (produced by running the reference itself, see
``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbhut_oracle.so")
_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U64 = ctypes.POINTER(ctypes.c_uint64)
_U8 = ctypes.POINTER(ctypes.c_uint8)


def build() -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, no FMA contraction)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "bhut_oracle.c")
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.bo_max_nodes.restype = ctypes.c_int64
        L.bo_max_nodes.argtypes = [ctypes.c_int64, ctypes.c_int]
        L.bo_build.restype = ctypes.c_int64
        L.bo_build.argtypes = [_D, _D, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _U64, _I64,
                               _D, _D, _D, _D, _I64, _I64, _I64, _I64, _U8]
        L.bo_topology.restype = ctypes.c_int64
        L.bo_topology.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int64,
                                  _I64, _I64, _I64, _I64, _U8]
        L.bo_aabb.argtypes = [_D, ctypes.c_int64, ctypes.c_int, _D, _D]
        L.bo_morton.argtypes = [_D, ctypes.c_int64, ctypes.c_int, _D, _D, _U64]
        L.bo_stable_argsort.argtypes = [_U64, ctypes.c_int64, _I64]
        L.bo_refit.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int64, _I64, _I64, _I64, _I64,
                               _U8, _I64, _D, _D, _D]
        L.bo_should_refit.restype = ctypes.c_int
        L.bo_should_refit.argtypes = [_D, ctypes.c_double, _D, ctypes.c_int64, ctypes.c_int]
        L.bo_accel.argtypes = [_D, _D, _D, _I64, _I64, _I64, _I64, _I64, ctypes.c_int64,
                               _D, _D, ctypes.c_int, _D, ctypes.c_int64, _I64,
                               ctypes.c_double, ctypes.c_double, ctypes.c_double, _D, _I64,
                               ctypes.c_int]
        L.bo_direct.argtypes = [_D, _D, ctypes.c_int64, ctypes.c_int, _D, ctypes.c_int64, _I64,
                                ctypes.c_double, ctypes.c_double, _D, ctypes.c_int]
        L.bo_tree_statistics.restype = ctypes.c_int
        L.bo_tree_statistics.argtypes = [_D, _D, _D, _I64, _I64, _I64, _I64, ctypes.c_int64,
                                         ctypes.c_int, _D, ctypes.c_int64, ctypes.c_double,
                                         _I64, ctypes.c_int]
        L.bo_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class OracleTree:
    """Same fields as the reference ``TreeData`` (bhut/tree/node.py:15-77)."""

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
    codes: np.ndarray
    dim: int
    leaf_size: int

    @property
    def num_nodes(self) -> int:
        return len(self.mass)


def morton_codes(pos: np.ndarray) -> np.ndarray:
    """Keys in input order: aabb + normalize_to_unit + morton_codes."""
    pos = _f64(pos)
    n, dim = pos.shape
    pmin = np.empty(dim)
    pmax = np.empty(dim)
    L = lib()
    L.bo_aabb(_p(pos, _D), n, dim, _p(pmin, _D), _p(pmax, _D))
    codes = np.empty(n, dtype=np.uint64)
    L.bo_morton(_p(pos, _D), n, dim, _p(pmin, _D), _p(pmax, _D), _p(codes, _U64))
    return codes


def stable_argsort(codes: np.ndarray) -> np.ndarray:
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    perm = np.empty(len(codes), dtype=np.int64)
    lib().bo_stable_argsort(_p(codes, _U64), len(codes), _p(perm, _I64))
    return perm


def topology(n: int, leaf_size: int):
    """(first_child, child_count, start, count, is_leaf) of build.py:110-212."""
    L = lib()
    mx = L.bo_max_nodes(n, leaf_size)
    fc = np.empty(mx, np.int64)
    cc = np.empty(mx, np.int64)
    st = np.empty(mx, np.int64)
    ct = np.empty(mx, np.int64)
    il = np.empty(mx, np.uint8)
    m = L.bo_topology(n, leaf_size, mx, _p(fc, _I64), _p(cc, _I64), _p(st, _I64), _p(ct, _I64),
                      _p(il, _U8))
    if m < 0:
        raise RuntimeError("node bound exceeded")
    return fc[:m], cc[:m], st[:m], ct[:m], il[:m].astype(bool)


def build_tree(pos: np.ndarray, masses: np.ndarray, leaf_size: int = 32) -> OracleTree:
    pos = _f64(pos)
    masses = _f64(masses)
    n, dim = pos.shape
    if n == 0:
        raise ValueError("Cannot build tree with zero particles")
    L = lib()
    mx = L.bo_max_nodes(n, leaf_size)
    codes = np.empty(n, np.uint64)
    perm = np.empty(n, np.int64)
    center = np.zeros((mx, dim))
    half = np.zeros(mx)
    mass = np.zeros(mx)
    com = np.zeros((mx, dim))
    fc = np.empty(mx, np.int64)
    cc = np.empty(mx, np.int64)
    st = np.empty(mx, np.int64)
    ct = np.empty(mx, np.int64)
    il = np.empty(mx, np.uint8)
    m = L.bo_build(_p(pos, _D), _p(masses, _D), n, dim, leaf_size, _p(codes, _U64), _p(perm, _I64),
                   _p(center, _D), _p(half, _D), _p(mass, _D), _p(com, _D), _p(fc, _I64),
                   _p(cc, _I64), _p(st, _I64), _p(ct, _I64), _p(il, _U8))
    if m < 0:
        raise RuntimeError(f"oracle build failed ({m})")
    return OracleTree(center[:m].copy(), half[:m].copy(), mass[:m].copy(), com[:m].copy(),
                      fc[:m].copy(), cc[:m].copy(), st[:m].copy(), ct[:m].copy(),
                      il[:m].astype(bool), perm, codes, dim, leaf_size)


def refit(tree: OracleTree, pos: np.ndarray, masses: np.ndarray) -> OracleTree:
    """refit_tree (refit.py:17-109): new mass/com, stale geometry and perm."""
    pos = _f64(pos)
    masses = _f64(masses)
    mass = tree.mass.copy()
    com = tree.com.copy()
    il = tree.is_leaf.astype(np.uint8)
    lib().bo_refit(_p(pos, _D), _p(masses, _D), tree.dim, tree.num_nodes,
                   _p(tree.first_child, _I64), _p(tree.child_count, _I64), _p(tree.start, _I64),
                   _p(tree.count, _I64), _p(il, _U8), _p(tree.perm, _I64),
                   _p(np.ascontiguousarray(tree.center), _D), _p(mass, _D), _p(com, _D))
    return OracleTree(tree.center.copy(), tree.half_size.copy(), mass, com,
                      tree.first_child.copy(), tree.child_count.copy(), tree.start.copy(),
                      tree.count.copy(), tree.is_leaf.copy(), tree.perm.copy(), tree.codes.copy(),
                      tree.dim, tree.leaf_size)


def should_refit(tree: OracleTree, pos: np.ndarray) -> bool:
    pos = _f64(pos)
    if pos.shape[0] != len(tree.perm) or pos.shape[1] != tree.dim:
        return False
    c0 = np.ascontiguousarray(tree.center[0])
    return bool(lib().bo_should_refit(_p(c0, _D), float(tree.half_size[0]), _p(pos, _D),
                                      pos.shape[0], tree.dim))


def accelerations(tree: OracleTree, pos: np.ndarray, masses: np.ndarray, *, theta: float,
                  softening: float, G: float = 1.0, targets: np.ndarray | None = None,
                  self_index: np.ndarray | None = None, nthreads: int = 0,
                  stats: bool = False):
    """Barnes-Hut accelerations.

    ``targets is None``: self accelerations (bh.py:428-482) for the particles
    ``self_index`` (all when None).  Otherwise external targets
    (bh.py:30-80).  With ``stats`` the per-target (visits, p2p, monopoles)
    counts are returned too.
    """
    pos = _f64(pos)
    masses = _f64(masses)
    n, dim = pos.shape
    if targets is None:
        idx = np.arange(n, dtype=np.int64) if self_index is None else np.ascontiguousarray(
            self_index, dtype=np.int64)
        nt = len(idx)
        tg = None
    else:
        tg = _f64(targets)
        idx = None
        nt = tg.shape[0]
    out = np.zeros((nt, dim))
    st = np.zeros((nt, 3), np.int64) if stats else None
    lib().bo_accel(_p(np.ascontiguousarray(tree.com), _D), _p(tree.half_size, _D),
                   _p(tree.mass, _D), _p(tree.first_child, _I64), _p(tree.child_count, _I64),
                   _p(tree.start, _I64), _p(tree.count, _I64), _p(tree.perm, _I64),
                   tree.num_nodes, _p(pos, _D), _p(masses, _D), dim, _p(tg, _D), nt,
                   _p(idx, _I64), float(theta), float(softening), float(G), _p(out, _D),
                   _p(st, _I64), int(nthreads))
    return (out, st) if stats else out


def direct_sum(pos: np.ndarray, masses: np.ndarray, *, softening: float, G: float = 1.0,
               targets: np.ndarray | None = None, self_index: np.ndarray | None = None,
               nthreads: int = 0) -> np.ndarray:
    pos = _f64(pos)
    masses = _f64(masses)
    n, dim = pos.shape
    if targets is None:
        idx = np.arange(n, dtype=np.int64) if self_index is None else np.ascontiguousarray(
            self_index, dtype=np.int64)
        nt = len(idx)
        tg = None
    else:
        tg = _f64(targets)
        idx = None
        nt = tg.shape[0]
    out = np.zeros((nt, dim))
    lib().bo_direct(_p(pos, _D), _p(masses, _D), n, dim, _p(tg, _D), nt, _p(idx, _I64),
                    float(softening), float(G), _p(out, _D), int(nthreads))
    return out


def tree_statistics(tree, targets: np.ndarray, theta: float = 0.5, nthreads: int = 0):
    """Totals (nodes_visited, particles_computed, monopoles_used) of
    compute_tree_statistics (bh.py:604-700) over ``targets``; ``tree`` is
    any object with the TreeData arrays."""
    tg = _f64(targets)
    i64 = lambda a: np.ascontiguousarray(a, dtype=np.int64)  # noqa: E731
    tot = np.zeros(3, np.int64)
    com = _f64(tree.com)
    rc = lib().bo_tree_statistics(_p(com, _D), _p(_f64(tree.half_size), _D),
                                  _p(_f64(tree.mass), _D), _p(i64(tree.first_child), _I64),
                                  _p(i64(tree.child_count), _I64), _p(i64(tree.start), _I64),
                                  _p(i64(tree.count), _I64), len(tree.mass), tg.shape[1],
                                  _p(tg, _D), tg.shape[0], float(theta), _p(tot, _I64),
                                  int(nthreads))
    if rc != 0:
        raise RuntimeError("tree statistics: traversal stack overflow")
    return tuple(int(v) for v in tot)


def num_threads() -> int:
    return int(lib().bo_num_threads())
