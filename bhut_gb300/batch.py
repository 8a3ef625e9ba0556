"""Batched form: many independent N-body systems per solve.

``BatchedSolver`` wraps the ``bhut_batch_*`` C ABI: systems are concatenated,
their trees are built with segmented kernels and one persistent traversal
kernel drains a global queue of (system, target chunk) tasks; the whole solve
can be replayed as one CUDA graph.  ``autotune`` picks the leaf size and the
targets per warp for a given batch by timing the candidates.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from .api import _is_cuda_tensor, _ptr, _sync_torch, _to_f64


def concat_systems(systems):
    """[(positions (n_i, dim), masses (n_i,)), ...] -> (positions, masses,
    offsets) with offsets[s] the first particle of system s."""
    sizes = [len(m) for _, m in systems]
    offsets = np.zeros(len(systems) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(sizes)
    pos = np.concatenate([np.asarray(p, dtype=np.float64) for p, _ in systems], axis=0)
    mass = np.concatenate([np.asarray(m, dtype=np.float64) for _, m in systems], axis=0)
    return np.ascontiguousarray(pos), np.ascontiguousarray(mass), offsets


class BatchedSolver:
    """Self accelerations of many systems in one solve."""

    def __init__(self, *, dim: int = 3, leaf_size: int = 32, form: str = "fp32",
                 criterion: str = "bh", targets_per_warp: int = 32, use_graph: bool = True,
                 stream: int | None = None, multipole: str = "mono", stack: str = "shared"):
        self.L = _lib.load()
        self.dim = dim
        self.leaf_size = leaf_size
        h = ctypes.c_void_p()
        _lib.check(self.L.bhut_batch_create(int(dim), int(leaf_size), stream, ctypes.byref(h)))
        self.h = h
        self.configure(form=form, criterion=criterion, targets_per_warp=targets_per_warp,
                       use_graph=use_graph, multipole=multipole, stack=stack)
        self.offsets = None
        self._keep = None

    def configure(self, *, form: str = "fp32", criterion: str = "bh", targets_per_warp: int = 32,
                  use_graph: bool = True, multipole: str = "mono",
                  stack: str = "shared") -> None:
        if form not in ("fp32", "fast"):
            raise ValueError(f"the batched solver runs form 'fp32' or 'fast', got {form!r}")
        if criterion not in _lib.CRITERIA:
            raise ValueError(f"criterion must be 'bh', got '{criterion}'")
        _lib.check(self.L.bhut_batch_configure(self.h, _lib.FORMS[form], _lib.CRITERIA[criterion],
                                               int(targets_per_warp), int(bool(use_graph))))
        if multipole not in _lib.MULTIPOLES:
            raise ValueError(f"multipole must be 'mono', got '{multipole}'")
        if multipole != "mono" and form != "fp32":
            raise ValueError(f"multipole must be 'mono', got '{multipole}' "
                         "(form='fp32' also accepts 'quad')")
        _lib.check(self.L.bhut_batch_set_multipole(self.h, _lib.MULTIPOLES[multipole]))
        if stack not in _lib.STACKS:
            raise ValueError(f"stack must be one of {sorted(_lib.STACKS)}, got {stack!r}")
        _lib.check(self.L.bhut_batch_set_stack(self.h, _lib.STACKS[stack]))
        self.form, self.criterion, self.multipole, self.stack = form, criterion, multipole, stack
        self.targets_per_warp, self.use_graph = targets_per_warp, use_graph

    def load(self, positions, masses, offsets) -> "BatchedSolver":
        pos = _to_f64(positions)
        m = _to_f64(masses)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        if tuple(pos.shape) != (int(off[-1]), self.dim) or tuple(m.shape) != (int(off[-1]),):
            raise ValueError("positions/masses do not match offsets")
        _sync_torch(pos, m)
        _lib.check(self.L.bhut_batch_load(self.h, _ptr(pos), _ptr(m), off.ctypes.data,
                                          len(off) - 1))
        self.offsets = off
        self._keep = (pos, m)
        self._cuda = _is_cuda_tensor(pos)
        return self

    def load_systems(self, systems) -> "BatchedSolver":
        return self.load(*concat_systems(systems))

    def solve(self, *, theta: float = 0.5, softening: float = 0.0, G: float = 1.0, out=None):
        if self.offsets is None:
            raise ValueError("load systems before solving")
        if theta < 0:
            raise ValueError(f"theta must be non-negative, got {theta}")
        if softening < 0:
            raise ValueError(f"softening must be non-negative, got {softening}")
        n = int(self.offsets[-1])
        if out is None:
            if self._cuda:
                import torch
                out = torch.empty((n, self.dim), dtype=torch.float64, device=self._keep[0].device)
            else:
                out = np.empty((n, self.dim))
        _lib.check(self.L.bhut_batch_solve(self.h, float(theta), float(softening), float(G),
                                           _ptr(out)))
        return out

    def split(self, acc):
        """Per-system views of a concatenated result."""
        return [acc[self.offsets[s]:self.offsets[s + 1]] for s in range(len(self.offsets) - 1)]

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self.L.bhut_batch_stats(self.h, ctypes.byref(a), ctypes.byref(b),
                                           ctypes.byref(c)))
        return a.value, b.value, c.value

    def traverse_ms(self) -> float:
        """Device time of the last solve's traversal kernel (CUDA events
        around its launch), milliseconds."""
        ms = ctypes.c_double()
        _lib.check(self.L.bhut_batch_traverse_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def info(self):
        v = [ctypes.c_int64() for _ in range(4)]
        _lib.check(self.L.bhut_batch_info(self.h, *[ctypes.byref(x) for x in v]))
        return {"systems": v[0].value, "particles": v[1].value, "nodes": v[2].value,
                "tasks": v[3].value}

    def close(self) -> None:
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.bhut_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batched_accelerations(systems, *, theta: float = 0.5, softening: float = 0.0,
                          G: float = 1.0, leaf_size: int = 32, form: str = "fp32",
                          criterion: str = "bh", targets_per_warp: int = 32,
                          multipole: str = "mono"):
    """Self accelerations of every (positions, masses) system; returns a list."""
    pos, m, off = concat_systems(systems)
    dim = pos.shape[1]
    sv = BatchedSolver(dim=dim, leaf_size=leaf_size, form=form, criterion=criterion,
                       multipole=multipole,
                       targets_per_warp=targets_per_warp, use_graph=False)
    try:
        sv.load(pos, m, off)
        acc = sv.solve(theta=theta, softening=softening, G=G)
        return [a.copy() for a in sv.split(acc)]
    finally:
        sv.close()


def autotune(positions, masses, offsets, *, theta: float, softening: float, G: float = 1.0,
             form: str = "fp32", criterion: str = "bh", leaf_sizes=(8, 16, 32, 64),
             targets_per_warp=(32, 16), stacks=("shared", "registers"), repeats: int = 2,
             multipole: str = "mono"):
    """Times every (leaf_size, targets_per_warp, stack placement) candidate on
    this batch (graph replay, warm) and returns (best config, {config:
    seconds})."""
    import torch
    pos = _to_f64(positions)
    m = _to_f64(masses)
    if not _is_cuda_tensor(pos):
        pos = torch.as_tensor(pos).cuda()
        m = torch.as_tensor(np.asarray(m)).cuda()
    dim = int(pos.shape[1])
    times = {}
    out = torch.empty((int(offsets[-1]), dim), dtype=torch.float64, device="cuda")
    for L in leaf_sizes:
        for tpw in targets_per_warp:
            if tpw != 32 and dim != 3:
                continue
            for stk in stacks:
                sv = BatchedSolver(dim=dim, leaf_size=L, form=form, criterion=criterion,
                                   targets_per_warp=tpw, use_graph=True, multipole=multipole,
                                   stack=stk)
                sv.load(pos, m, offsets)
                best = float("inf")
                for r in range(repeats + 1):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    sv.solve(theta=theta, softening=softening, G=G, out=out)
                    torch.cuda.synchronize()
                    if r:
                        best = min(best, time.perf_counter() - t0)
                sv.close()
                times[(L, tpw, stk)] = best
    best = min(times, key=times.get)
    return {"leaf_size": best[0], "targets_per_warp": best[1], "stack": best[2]}, times


def main():
    """Times the batched solver on seeded Plummer systems:

        python -m bhut_gb300.batch [--nsys 2048] [--nmin 256] [--nmax 65536]
            [--leaf 16] [--tpw 32] [--form fp32] [--multipole mono] [--solves 3]

    prints one JSON line (ms per solve, systems/s, accels/s)."""
    import argparse
    import json

    import torch

    from . import workloads
    ap = argparse.ArgumentParser()
    ap.add_argument("--nsys", type=int, default=2048)
    ap.add_argument("--nmin", type=int, default=256)
    ap.add_argument("--nmax", type=int, default=65536)
    ap.add_argument("--leaf", type=int, default=16)
    ap.add_argument("--tpw", type=int, default=32)
    ap.add_argument("--form", default="fp32")
    ap.add_argument("--criterion", default="bh")
    ap.add_argument("--multipole", default="mono")
    ap.add_argument("--stack", default="shared")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--softening", type=float, default=0.01)
    ap.add_argument("--solves", type=int, default=3)
    ap.add_argument("--seed", type=int, default=11)
    a = ap.parse_args()
    pos, m, off = concat_systems(workloads.plummer_batch(a.nsys, a.nmin, a.nmax, seed=a.seed))
    pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
    sv = BatchedSolver(leaf_size=a.leaf, form=a.form, criterion=a.criterion,
                       targets_per_warp=a.tpw, use_graph=True, multipole=a.multipole,
                       stack=a.stack)
    sv.load(pd, md, off)
    out = torch.empty_like(pd)
    sv.solve(theta=a.theta, softening=a.softening, out=out)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(a.solves):
        sv.solve(theta=a.theta, softening=a.softening, out=out)
    ev1.record()
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / a.solves
    p2p, m2p, visits = sv.stats()
    sv.close()
    print(json.dumps({"systems": a.nsys, "particles": int(off[-1]), "ms_per_solve": ms,
                      "systems_per_s": a.nsys / ms * 1e3, "accels_per_s": off[-1] / ms * 1e3,
                      "p2p": p2p, "m2p": m2p, "visits": visits, "leaf": a.leaf, "tpw": a.tpw,
                      "form": a.form, "multipole": a.multipole, "stack": a.stack}), flush=True)


if __name__ == "__main__":
    main()
