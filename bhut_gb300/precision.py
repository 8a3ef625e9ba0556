"""Accuracy reporting and leaf-size autotuning for the FP32 precision form.

Every FP32 result can carry its relative-error distribution against an FP64
direct sum evaluated on the GPU at a seeded sample of targets
(``sampled_errors``).  ``autotune_leaf_size`` times the traversal for each
candidate leaf size on the actual system and keeps the fastest.
"""
from __future__ import annotations

import time

import numpy as np

from . import api


def error_distribution(acc, ref) -> dict:
    """Per-target relative error |a - a_ref| / |a_ref|: median, p90, p99, max,
    plus the relative L2 error over all targets."""
    acc = np.asarray(acc, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    num = np.linalg.norm(acc - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    ok = den > 0
    rel = num[ok] / den[ok]
    if rel.size == 0:
        return {"median": 0.0, "p90": 0.0, "p99": 0.0, "max": 0.0, "rel_l2": 0.0, "n": 0}
    return {"median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
            "p99": float(np.percentile(rel, 99)), "max": float(rel.max()),
            "rel_l2": float(np.linalg.norm(acc - ref) / max(np.linalg.norm(ref), 1e-300)),
            "n": int(rel.size)}


def sample_indices(n: int, n_sample: int = 8192, seed: int = 0) -> np.ndarray:
    return np.sort(np.random.default_rng(seed).choice(n, min(n, n_sample), replace=False))


def direct_reference(positions, masses, idx, *, softening: float, G: float = 1.0) -> np.ndarray:
    """FP64 direct sum at the particles ``idx`` (their own zero-displacement
    term contributes nothing), evaluated on the GPU."""
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    return np.asarray(api.direct_accelerations(pos, masses, softening=softening, G=G,
                                               targets=pos[idx]))


def sampled_errors(positions, masses, acc, *, softening: float, G: float = 1.0,
                   n_sample: int = 8192, seed: int = 0, reference=None) -> dict:
    """Error distribution of self accelerations ``acc`` against the FP64
    direct sum on ``n_sample`` seeded targets."""
    idx = sample_indices(len(positions), n_sample, seed)
    ref = direct_reference(positions, masses, idx, softening=softening, G=G) \
        if reference is None else reference
    return error_distribution(np.asarray(acc)[idx], ref)


def accelerations_with_errors(positions, masses, *, theta: float = 0.5, softening: float = 0.0,
                              G: float = 1.0, form: str = "fp32", criterion: str = "bh",
                              multipole: str = "mono", leaf_size: int = 32,
                              n_sample: int = 1024, seed: int = 0):
    """Self accelerations together with their relative-error distribution
    against the FP64 direct sum at ``n_sample`` seeded targets:
    returns (accelerations, distribution)."""
    acc = api.accelerations(positions, masses, theta=theta, softening=softening, G=G,
                            form=form, criterion=criterion, multipole=multipole,
                            leaf_size=leaf_size)
    pos = np.asarray(api._host(positions))
    m = np.asarray(api._host(masses))
    host = acc.cpu().numpy() if api._is_torch(acc) else np.asarray(acc)
    dist = sampled_errors(pos, m, host, softening=softening, G=G, n_sample=n_sample, seed=seed)
    return acc, dist


def batched_with_errors(systems, *, theta: float = 0.5, softening: float = 0.0, G: float = 1.0,
                        form: str = "fp32", criterion: str = "bh", multipole: str = "mono",
                        leaf_size: int = 32, n_sample: int = 256, seed: int = 0):
    """Batched solve of [(positions, masses), ...]; every system's result
    comes with its own error distribution against the FP64 direct sum at up
    to ``n_sample`` seeded targets: returns [(accelerations, distribution)]."""
    from . import batch
    accs = batch.batched_accelerations(systems, theta=theta, softening=softening, G=G,
                                       leaf_size=leaf_size, form=form, criterion=criterion,
                                       multipole=multipole)
    return [(a, sampled_errors(np.asarray(p), np.asarray(m), a, softening=softening, G=G,
                               n_sample=n_sample, seed=seed))
            for (p, m), a in zip(systems, accs)]


def autotune_leaf_size(positions, masses, *, theta: float, softening: float, G: float = 1.0,
                       form: str = "fp32", criterion: str = "bh", multipole: str = "mono",
                       candidates=(8, 16, 32, 64), repeats: int = 2) -> tuple[int, dict]:
    """Builds a tree per candidate leaf size and times build + self traversal;
    returns (best leaf size, {leaf_size: seconds})."""
    import torch

    def dev(a):
        if isinstance(a, torch.Tensor):
            return a.to(device="cuda", dtype=torch.float64).contiguous()
        return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    pos = dev(positions)
    m = dev(masses)
    times = {}
    for L in candidates:
        tree = api.Tree(pos, m, leaf_size=L, form=form, criterion=criterion,
                        multipole=multipole)
        best = float("inf")
        for r in range(repeats + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tree.rebuild(pos, m)
            tree.accelerations(theta=theta, softening=softening, G=G)
            torch.cuda.synchronize()
            if r:
                best = min(best, time.perf_counter() - t0)
        tree.close()
        times[L] = best
    return min(times, key=times.get), times
