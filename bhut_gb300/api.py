"""Public API: a drop-in for bhut 0.1.0's ``accelerations`` and ``Tree``.

Signatures, argument meaning, validation order and error messages follow
bhut/api.py (file:line cited per function).  The arithmetic runs in
libbhut_gb300.so through the C ABI of include/bhut_gb300.h; this module only
validates, converts and marshals.  Inputs may be anything ``np.asarray``
accepts, or torch tensors: CUDA tensors are passed to the engine zero-copy
and the result comes back as a CUDA tensor on the same device.

One keyword is added to both entry points: ``form`` selects the traversal
arithmetic -- ``"exact"`` (FP64; pair terms bit-identical to the reference's
Numba loop), ``"fast"`` (FP64-accurate float-float arithmetic on the FP32
pipe) or ``"fp32"`` (the FP32/Kahan precision form).  ``criterion`` accepts,
besides the reference's ``"bh"``, ``"bh_offset"`` (open when
|x - com| < size/theta + |com - box centre|), available with ``form="fp32"``;
``multipole`` accepts, besides ``"mono"``, ``"quad"`` (monopole plus traceless
quadrupole per node), also with ``form="fp32"`` only.
"""
from __future__ import annotations

import ctypes
from typing import Any, Optional

import numpy as np

from . import _lib
from .tree.node import TreeData

DEFAULT_FORM = "fast"


# ---------------------------------------------------------------------------
# array plumbing
# ---------------------------------------------------------------------------
def _is_torch(x) -> bool:
    return type(x).__module__.split(".")[0] == "torch" and hasattr(x, "data_ptr")


def _is_cuda_tensor(x) -> bool:
    return _is_torch(x) and bool(getattr(x, "is_cuda", False))


def _torch():
    import torch
    return torch


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if _is_torch(a):
        return a.data_ptr()
    return a.ctypes.data


def _sync_torch(*arrays) -> None:
    if any(_is_cuda_tensor(a) for a in arrays if a is not None):
        _torch().cuda.current_stream().synchronize()


def _to_f64(x):
    """np.asarray(x, dtype=float64), keeping CUDA tensors on their device."""
    if _is_cuda_tensor(x):
        t = x.detach()
        if t.dtype != _torch().float64:
            t = t.to(_torch().float64)
        return t.contiguous()
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def _shape(a):
    return tuple(a.shape)


def _empty_like_out(ref, shape):
    if _is_cuda_tensor(ref):
        return _torch().empty(shape, dtype=_torch().float64, device=ref.device)
    return np.empty(shape, dtype=np.float64)


# ---------------------------------------------------------------------------
# validation (bhut/api.py:84-152, bhut/backends/base.py:102-166)
# ---------------------------------------------------------------------------
def _validate_dimensions(dim: int) -> None:
    if dim not in (2, 3):
        raise ValueError(f"dim must be 2 or 3, got {dim}")


def _check_backend(array, backend: str) -> str:
    """get_namespace (bhut/backends/base.py:102-166) without the Dask path."""
    if not _is_cuda_tensor(array):
        np.asarray(array)
    if backend == "auto":
        return "numpy"
    if backend == "numpy":
        return "numpy"
    if backend == "dask":
        raise ValueError("Unsupported backend: dask. The Dask chunking path is not part of the "
                         "GB300 engine; pass NumPy arrays or torch tensors")
    raise ValueError(f"Unsupported backend: {backend}. Supported: 'numpy', 'dask', 'auto'")


def _validate_accelerations_inputs(positions, masses, *, dim, softening, theta, G, leaf_size):
    """bhut/api.py:90-152."""
    _validate_dimensions(dim)
    positions = _to_f64(positions)
    masses = _to_f64(masses)
    if len(_shape(positions)) != 2:
        raise ValueError(f"positions must be 2D array, got shape {_shape(positions)}")
    if len(_shape(masses)) != 1:
        raise ValueError(f"masses must be 1D array, got shape {_shape(masses)}")
    N, actual_dim = _shape(positions)
    if actual_dim != dim:
        raise ValueError(f"positions has {actual_dim} dimensions but dim={dim}")
    if _shape(masses)[0] != N:
        raise ValueError(f"positions has {N} particles but masses has {_shape(masses)[0]} elements")
    if np.isscalar(softening):
        softening = float(softening)
        if softening < 0:
            raise ValueError(f"softening must be non-negative, got {softening}")
    else:
        softening = _host(softening)
        if len(softening.shape) != 1:
            raise ValueError(f"softening array must be 1D, got shape {softening.shape}")
        if softening.shape[0] != N:
            raise ValueError(f"softening array has {softening.shape[0]} elements but need {N}")
        if np.any(softening < 0):
            raise ValueError("all softening values must be non-negative")
    if theta < 0:
        raise ValueError(f"theta must be non-negative, got {theta}")
    if leaf_size <= 0:
        raise ValueError(f"leaf_size must be positive, got {leaf_size}")
    return positions, masses, softening


def _host(x) -> np.ndarray:
    if _is_torch(x):
        return x.detach().cpu().numpy().astype(np.float64)
    return np.asarray(x, dtype=np.float64)


def _scalar_softening(softening, n: int) -> float:
    """evaluate_accelerations (bhut/api.py:400-418): uniform arrays collapse to
    a scalar, anything else is rejected."""
    s = np.asarray(_host(softening) if _is_torch(softening) else softening, dtype=np.float64)
    if s.ndim > 1:
        raise ValueError("Softening must be scalar or 1D array")
    if s.ndim == 1 and len(s) != n:
        raise ValueError("Softening array length must match number of particles")
    if np.any(s < 0):
        raise ValueError("Softening must be non-negative")
    if s.ndim == 1:
        if not np.allclose(s, s[0]):
            raise ValueError("Variable softening per particle not yet implemented")
        return float(s[0])
    return float(s)


def _form_code(form: str) -> int:
    try:
        return _lib.FORMS[form]
    except KeyError:
        raise ValueError(f"form must be one of {sorted(_lib.FORMS)}, got {form!r}") from None


def _criterion_code(criterion: str, form: str) -> int:
    if criterion not in _lib.CRITERIA:
        raise ValueError(f"criterion must be 'bh', got '{criterion}'")
    if criterion != "bh" and form != "fp32":
        raise ValueError(f"criterion '{criterion}' is available with form='fp32' only")
    return _lib.CRITERIA[criterion]


def _multipole_code(multipole: str, form: str) -> int:
    if multipole not in _lib.MULTIPOLES:
        raise ValueError(f"multipole must be 'mono', got '{multipole}'")
    if multipole != "mono" and form != "fp32":
        raise ValueError(f"multipole must be 'mono', got '{multipole}' "
                         "(form='fp32' also accepts 'quad')")
    return _lib.MULTIPOLES[multipole]


# ---------------------------------------------------------------------------
# TreeData (bhut/tree/node.py:15-181) lives in bhut_gb300/tree/node.py, the
# reference's module path; the engine exports its device tree into it.
# ---------------------------------------------------------------------------


class _Handle:
    """Owns one bhut_tree* of the C ABI."""

    def __init__(self, dim: int, leaf_size: int, stream: int | None = None):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self.L.bhut_tree_create(int(dim), int(leaf_size), stream, ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.bhut_tree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_form(self, form: str, criterion: str = "bh", multipole: str = "mono") -> None:
        _lib.check(self.L.bhut_tree_set_form(self.h, _form_code(form)))
        _lib.check(self.L.bhut_tree_set_criterion(self.h, _criterion_code(criterion, form)))
        _lib.check(self.L.bhut_tree_set_multipole(self.h, _multipole_code(multipole, form)))

    def build(self, pos, m) -> None:
        _sync_torch(pos, m)
        _lib.check(self.L.bhut_tree_build(self.h, _ptr(pos), _ptr(m), int(_shape(pos)[0])))

    def refit(self, pos, m) -> bool:
        _sync_torch(pos, m)
        rebuilt = ctypes.c_int(0)
        _lib.check(self.L.bhut_tree_refit(self.h, _ptr(pos), _ptr(m), int(_shape(pos)[0]),
                                          ctypes.byref(rebuilt)))
        return bool(rebuilt.value)

    def rebuild(self, pos, m) -> None:
        _sync_torch(pos, m)
        _lib.check(self.L.bhut_tree_rebuild(self.h, _ptr(pos), _ptr(m), int(_shape(pos)[0])))

    def stats(self):
        """(pair evaluations, monopole evaluations, node visits) of the last
        traversal, summed over targets."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self.L.bhut_tree_stats(self.h, ctypes.byref(a), ctypes.byref(b),
                                          ctypes.byref(c)))
        return a.value, b.value, c.value

    def fallbacks(self):
        """(exact opening decisions, FP64 pairs) of the last fast traversal."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self.L.bhut_tree_fallbacks(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def info(self):
        n, m = ctypes.c_int64(), ctypes.c_int64()
        d, L = ctypes.c_int(), ctypes.c_int()
        _lib.check(self.L.bhut_tree_info(self.h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(d),
                                         ctypes.byref(L)))
        return n.value, m.value, d.value, L.value

    def accel_self(self, theta, eps, G, out) -> None:
        _sync_torch(out)
        _lib.check(self.L.bhut_tree_accel_self(self.h, float(theta), float(eps), float(G),
                                               _ptr(out)))

    def accel_targets(self, targets, theta, eps, G, out) -> None:
        _sync_torch(targets, out)
        _lib.check(self.L.bhut_tree_accel_targets(self.h, _ptr(targets), int(_shape(targets)[0]),
                                                  float(theta), float(eps), float(G), _ptr(out)))

    def import_tree(self, td: "TreeData", pos, m) -> None:
        """Loads a TreeData and the particles it indexes (bhut_tree_import)."""
        i64 = lambda a: np.ascontiguousarray(np.asarray(a), dtype=np.int64)  # noqa: E731
        f64 = lambda a: np.ascontiguousarray(np.asarray(a), dtype=np.float64)  # noqa: E731
        keep = (i64(td.first_child), i64(td.child_count), i64(td.start), i64(td.count),
                i64(td.perm), f64(td.center), f64(td.half_size), f64(td.mass), f64(td.com))
        _sync_torch(pos, m)
        _lib.check(self.L.bhut_tree_import(self.h, _ptr(pos), _ptr(m), int(_shape(pos)[0]),
                                           *[a.ctypes.data for a in keep], len(keep[7])))

    def refit_only(self, pos, m) -> None:
        _sync_torch(pos, m)
        _lib.check(self.L.bhut_tree_refit_only(self.h, _ptr(pos), _ptr(m), int(_shape(pos)[0])))

    def export(self) -> TreeData:
        n, m, dim, L = self.info()
        center = np.empty((m, dim))
        half = np.empty(m)
        mass = np.empty(m)
        com = np.empty((m, dim))
        fc = np.empty(m, np.int64)
        cc = np.empty(m, np.int64)
        st = np.empty(m, np.int64)
        ct = np.empty(m, np.int64)
        il = np.empty(m, np.uint8)
        perm = np.empty(n, np.int64)
        _lib.check(self.L.bhut_tree_export(self.h, *[a.ctypes.data for a in
                                                      (center, half, mass, com, fc, cc, st, ct, il,
                                                       perm)]))
        return TreeData(center, half, mass, com, fc.astype(np.intp), cc.astype(np.intp),
                        st.astype(np.intp), ct.astype(np.intp), il.astype(bool),
                        perm.astype(np.intp), dim, L)


# ---------------------------------------------------------------------------
# functional API (bhut/api.py:254-364)
# ---------------------------------------------------------------------------
def accelerations(
    positions,
    masses,
    *,
    theta: float = 0.5,
    softening: Any = 0.0,
    G: float = 1.0,
    dim: int = 3,
    backend: str = "auto",
    leaf_size: int = 32,
    criterion: str = "bh",
    multipole: str = "mono",
    form: str | None = None,
):
    """Gravitational self-accelerations with the Barnes-Hut algorithm.

    Same contract as bhut.accelerations (bhut/api.py:254-364): builds the
    Morton count-split tree of the particles and evaluates the softened
    monopole/P2P traversal at every particle, skipping self-interaction.
    Returns a float64 (N, dim) array (a CUDA tensor for CUDA tensor input).
    """
    if criterion not in _lib.CRITERIA:
        raise ValueError(f"criterion must be 'bh', got '{criterion}'")
    if multipole not in _lib.MULTIPOLES:
        raise ValueError(f"multipole must be 'mono', got '{multipole}'")
    _criterion_code(criterion, form or DEFAULT_FORM)
    _multipole_code(multipole, form or DEFAULT_FORM)
    _check_backend(positions, backend)
    positions, masses, softening = _validate_accelerations_inputs(
        positions, masses, dim=dim, softening=softening, theta=theta, G=G, leaf_size=leaf_size)
    n = _shape(positions)[0]
    if n == 0:
        raise ValueError("Cannot build tree with zero particles")
    eps = _scalar_softening(softening, n)
    if theta < 0:
        raise ValueError("Opening angle theta must be non-negative")
    h = _Handle(dim, leaf_size)
    try:
        h.set_form(form or DEFAULT_FORM, criterion, multipole)
        h.build(positions, masses)
        out = _empty_like_out(positions, (n, dim))
        h.accel_self(theta, eps, G, out)
    finally:
        h.close()
    return out


def accelerations_chunks(position_chunks, mass_chunks, *, theta: float = 0.5,
                         softening: float = 0.0, G: float = 1.0, dim: int = 3,
                         leaf_size: int = 32, form: str | None = None) -> list:
    """The chunked self-acceleration path of bhut/api.py:28-78 without Dask:
    the tree is built once over all chunks, each chunk's particles are then
    evaluated as targets (no self skip, as the reference's map_blocks call of
    barnes_hut_accelerations_targets; a particle's own zero-distance pair
    contributes nothing) and the results come back in the same chunks."""
    pos = [_to_f64(c) for c in position_chunks]
    ms = [_to_f64(c) for c in mass_chunks]
    if len(pos) != len(ms):
        raise ValueError("position and mass chunk counts differ")
    if pos and _is_cuda_tensor(pos[0]):
        torch = _torch()
        p_all, m_all = torch.cat(pos), torch.cat([m.to(pos[0].device) for m in ms])
    else:
        p_all = np.concatenate([np.asarray(_host(c)) for c in pos])
        m_all = np.concatenate([np.asarray(_host(c)) for c in ms])
    tree = Tree(p_all, m_all, leaf_size=leaf_size, dim=dim, form=form).build()
    try:
        return tree.accelerations_chunks(pos, theta=theta, softening=softening, G=G)
    finally:
        tree.close()


def build_tree(positions, masses, *, leaf_size: int, backend: str, dim: int) -> TreeData:
    """bhut/api.py:155-191: build and return the TreeData arrays."""
    _check_backend(positions, backend)
    positions = _to_f64(positions)
    masses = _to_f64(masses)
    h = _Handle(dim, leaf_size)
    try:
        h.build(positions, masses)
        return h.export()
    finally:
        h.close()


# ---------------------------------------------------------------------------
# object API (bhut/api.py:432-786)
# ---------------------------------------------------------------------------
class Tree:
    """Barnes-Hut tree resident in GPU memory (bhut/api.py:432-786).

    Attributes as in the reference: ``positions``, ``masses``, ``dim``,
    ``leaf_size``, ``backend``, ``_tree`` (TreeData, exported from the device
    on access) and ``_is_built``.
    """

    def __init__(self, positions, masses, *, leaf_size: int = 32, backend: str = "auto",
                 dim: int = 3, form: str | None = None, criterion: str = "bh",
                 multipole: str = "mono"):
        _validate_dimensions(dim)
        self.positions, self.masses, _ = _validate_accelerations_inputs(
            positions, masses, dim=dim, softening=0.0, theta=0.5, G=1.0, leaf_size=leaf_size)
        self.dim = dim
        self.leaf_size = leaf_size
        self.backend = backend
        self._is_built = False
        self._tree_cache: TreeData | None = None
        self._handle: _Handle | None = None
        self._form = form or DEFAULT_FORM
        _form_code(self._form)
        self._criterion = criterion
        _criterion_code(criterion, self._form)
        self._multipole = multipole
        _multipole_code(multipole, self._form)
        _check_backend(self.positions, backend)

    # -- reference attribute ``_tree``: None until built --------------------
    @property
    def _tree(self) -> TreeData | None:
        if not self._is_built or self._handle is None:
            return None
        if self._tree_cache is None:
            self._tree_cache = self._handle.export()
        return self._tree_cache

    @_tree.setter
    def _tree(self, value) -> None:
        if value is None:
            self._is_built = False
            self._tree_cache = None
        else:
            raise AttributeError("_tree is derived from the device tree")

    def close(self) -> None:
        """Release the device memory of this tree."""
        if self._handle is not None:
            self._handle.close()
            self._handle = None
        self._is_built = False
        self._tree_cache = None

    def set_form(self, form: str, criterion: str = "bh", multipole: str = "mono") -> "Tree":
        """Traversal arithmetic ("exact", "fast", "fp32") and, for "fp32",
        the opening criterion ("bh" or "bh_offset") and node expansion
        ("mono" or "quad")."""
        _form_code(form)
        _criterion_code(criterion, form)
        _multipole_code(multipole, form)
        self._form = form
        self._criterion = criterion
        self._multipole = multipole
        return self

    def build(self) -> "Tree":
        """bhut/api.py:497-511."""
        if _shape(self.positions)[0] == 0:
            raise ValueError("Cannot build tree with zero particles")
        if self._handle is None:
            self._handle = _Handle(self.dim, self.leaf_size)
        self._tree_cache = None
        self._is_built = False
        self._handle.build(self.positions, self.masses)
        self._is_built = True
        return self

    def refit(self, new_positions, new_masses=None) -> "Tree":
        """bhut/api.py:513-562 (falls back to rebuild as refit.py:195-251)."""
        if not self._is_built or self._handle is None:
            raise ValueError("Tree must be built before refitting. Call build() first.")
        if new_masses is None:
            new_masses = self.masses
        new_positions, new_masses, _ = _validate_accelerations_inputs(
            new_positions, new_masses, dim=self.dim, softening=0.0, theta=0.5, G=1.0,
            leaf_size=self.leaf_size)
        if _shape(new_positions)[0] == 0:
            raise ValueError("Cannot build tree with zero particles")
        self._tree_cache = None
        self._handle.refit(new_positions, new_masses)
        self.positions = new_positions
        self.masses = new_masses
        return self

    def rebuild(self, new_positions, new_masses=None) -> "Tree":
        """bhut/api.py:564-606."""
        if new_masses is None:
            new_masses = self.masses
        new_positions, new_masses, _ = _validate_accelerations_inputs(
            new_positions, new_masses, dim=self.dim, softening=0.0, theta=0.5, G=1.0,
            leaf_size=self.leaf_size)
        if _shape(new_positions)[0] == 0:
            raise ValueError("Cannot build tree with zero particles")
        if self._handle is None:
            self._handle = _Handle(self.dim, self.leaf_size)
        # the device rejects non-finite input before touching the built tree,
        # so a failed rebuild leaves this Tree as it was
        self._handle.build(new_positions, new_masses)
        self.positions = new_positions
        self.masses = new_masses
        self._tree_cache = None
        self._is_built = True
        return self

    def accelerations(self, targets=None, *, theta: float = 0.5, softening: Any = 0.0,
                      G: float = 1.0):
        """bhut/api.py:608-688: self accelerations, or at external targets."""
        if not self._is_built:
            raise ValueError("Tree must be built before evaluating accelerations")
        if targets is None:
            return self.evaluate_accelerations(softening, theta, G)
        targets = _to_f64(targets)
        if len(_shape(targets)) != 2:
            raise ValueError(f"targets must be 2D array, got shape {_shape(targets)}")
        if _shape(targets)[1] != self.dim:
            raise ValueError(f"targets has {_shape(targets)[1]} dimensions but tree has {self.dim}")
        M = _shape(targets)[0]
        if not np.isscalar(softening):
            s = _host(softening)
            if s.shape != (M,):
                raise ValueError(f"softening array shape {s.shape} does not match "
                                 f"targets shape ({M},)")
            eps = _scalar_softening(s, M)
        else:
            eps = float(softening)
            if eps < 0:
                raise ValueError(f"softening must be non-negative, got {eps}")
        if theta < 0:
            raise ValueError(f"theta must be non-negative, got {theta}")
        out = _empty_like_out(targets, (M, self.dim))
        if M:
            self._handle.set_form(self._form, self._criterion, self._multipole)
            self._handle.accel_targets(targets, theta, eps, G, out)
        return out

    def accelerations_chunks(self, target_chunks, *, theta: float = 0.5, softening: float = 0.0,
                             G: float = 1.0) -> list:
        """Chunks in, chunks out: the map_blocks path of bhut/api.py:690-731
        without Dask.  The chunks are evaluated in ONE traversal launch over
        their concatenation (each target's result does not depend on which
        other targets share the launch) and the result is returned split
        into chunks of the same lengths, as CUDA tensors for CUDA chunks."""
        chunks = [_to_f64(c) for c in target_chunks]
        if not chunks:
            return []
        for c in chunks:
            if len(_shape(c)) != 2 or _shape(c)[1] != self.dim:
                raise ValueError(f"target chunk has shape {_shape(c)}, expected (k, {self.dim})")
        sizes = [_shape(c)[0] for c in chunks]
        if _is_cuda_tensor(chunks[0]):
            torch = _torch()
            allt = torch.cat([c.to(chunks[0].device) for c in chunks])
            out = self.accelerations(allt, theta=theta, softening=softening, G=G)
            return list(torch.split(out, sizes))
        allt = np.concatenate([np.asarray(_host(c)) for c in chunks])
        out = self.accelerations(allt, theta=theta, softening=softening, G=G)
        return np.split(out, np.cumsum(sizes)[:-1])

    def evaluate_accelerations(self, softening, theta: float = 0.5, G: float = 1.0):
        """bhut/api.py:733-786."""
        if not self._is_built or self._handle is None:
            raise RuntimeError("Tree not built. Call build() first.")
        if not isinstance(softening, (int, float)):
            raise ValueError("Only scalar softening is currently supported")
        if softening < 0:
            raise ValueError("Softening must be non-negative")
        if theta < 0:
            raise ValueError("Opening angle theta must be non-negative")
        n = _shape(self.positions)[0]
        out = _empty_like_out(self.positions, (n, self.dim))
        self._handle.set_form(self._form, self._criterion, self._multipole)
        self._handle.accel_self(theta, float(softening), G, out)
        return out

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# building blocks exposed for parity checks
# ---------------------------------------------------------------------------
def morton_keys(positions) -> np.ndarray:
    """Morton keys in input order (bbox.py + morton.py:48-102)."""
    pos = _to_f64(positions)
    n, dim = _shape(pos)
    keys = np.empty(n, np.uint64)
    _sync_torch(pos)
    _lib.check(_lib.load().bhut_morton_keys(_ptr(pos), n, dim, keys.ctypes.data, None))
    return keys


def morton_argsort(positions):
    """(sorted keys, stable permutation) as sort_by_morton (morton.py:105-147)."""
    pos = _to_f64(positions)
    n, dim = _shape(pos)
    keys = np.empty(n, np.uint64)
    perm = np.empty(n, np.int64)
    _sync_torch(pos)
    _lib.check(_lib.load().bhut_morton_argsort(_ptr(pos), n, dim, keys.ctypes.data,
                                               perm.ctypes.data, None))
    return keys, perm


def direct_accelerations(positions, masses, *, softening: float = 0.0, G: float = 1.0,
                         targets=None):
    """FP64 direct sum on the GPU (self accelerations when targets is None)."""
    pos = _to_f64(positions)
    m = _to_f64(masses)
    n, dim = _shape(pos)
    tg = None if targets is None else _to_f64(targets)
    mt = n if tg is None else _shape(tg)[0]
    out = _empty_like_out(pos, (mt, dim))
    _sync_torch(pos, m, tg, out)
    _lib.check(_lib.load().bhut_direct_accelerations(_ptr(pos), _ptr(m), n, dim, _ptr(tg), mt,
                                                     float(softening), float(G), _ptr(out), None))
    return out


def compute_tree_statistics(tree, positions, theta: float = 0.5) -> dict:
    """bhut/traverse/bh.py:604-700 on the GPU: average nodes visited,
    particles computed and monopoles used per target, and their total.

    ``tree`` is a TreeData (from ``Tree._tree`` or ``build_tree``) or a built
    ``Tree``; ``positions`` are the targets (N, dim).  Counting follows the
    reference exactly: every popped node is a visit, a visited non-empty leaf
    counts ``count - 1`` particles whether or not the target lies in it, an
    accepted internal node counts one monopole.
    """
    if isinstance(tree, Tree):
        tree = tree._tree
        if tree is None:
            raise RuntimeError("Tree not built. Call build() first.")
    pos = np.ascontiguousarray(_host(positions), dtype=np.float64)
    n_particles = len(pos)
    dim = pos.shape[1] if pos.ndim == 2 else tree.dim
    i64 = lambda a: np.ascontiguousarray(a, dtype=np.int64)  # noqa: E731
    arrays = [np.ascontiguousarray(tree.com, dtype=np.float64),
              np.ascontiguousarray(tree.half_size, dtype=np.float64),
              np.ascontiguousarray(tree.mass, dtype=np.float64),
              i64(tree.first_child), i64(tree.child_count), i64(tree.start), i64(tree.count)]
    totals = np.zeros(3, dtype=np.int64)
    _lib.check(_lib.load().bhut_tree_statistics(
        *[a.ctypes.data for a in arrays], len(arrays[2]), int(dim), pos.ctypes.data,
        n_particles, float(theta), None, totals.ctypes.data))
    nodes, parts, monos = (int(v) for v in totals)
    return {
        "avg_nodes_visited": nodes / n_particles,
        "avg_particles_computed": parts / n_particles,
        "avg_monopoles_used": monos / n_particles,
        "total_operations": parts + monos,
    }
