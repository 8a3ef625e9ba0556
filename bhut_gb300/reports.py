"""Measurement reports for the engine's forms beyond the plain FP64 path.

    python -m bhut_gb300.reports precision [--n 4000000] [--sample 8192]

``precision``: the galaxy model (70 % exponential disc, 30 % Hernquist bulge,
equal masses), softening 0.005, theta in {0.3, 0.5, 0.7}.  For each theta the
leaf size of the FP32 form is autotuned over {8, 16, 32, 64}; the FP32/Kahan
self accelerations and the FP64-accurate ones (form "fast", same leaf size)
are timed, and both are compared with an FP64 direct sum on seeded sampled
targets.  One JSON line per theta.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import api, precision, workloads


def _timed_solve(tree, theta, eps, G, reps=2):
    import torch
    best = float("inf")
    acc = None
    for r in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        acc = tree.accelerations(theta=theta, softening=eps, G=G)
        torch.cuda.synchronize()
        if r:
            best = min(best, time.perf_counter() - t0)
    return acc, best


def _log(msg):
    print(f"[{time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def precision_report(n: int = 4_000_000, n_sample: int = 8192, thetas=(0.3, 0.5, 0.7),
                     eps: float = 0.005, G: float = 1.0, seed: int = 7, criterion: str = "bh"):
    import torch
    pos, m = workloads.galaxy(n, seed=seed)
    _log(f"galaxy N={n} generated")
    idx = precision.sample_indices(n, n_sample, seed=seed + 1)
    t0 = time.perf_counter()
    ref = precision.direct_reference(pos, m, idx, softening=eps, G=G)
    t_direct = time.perf_counter() - t0
    _log(f"direct sum on {len(idx)} targets: {t_direct:.2f} s")
    pd = torch.as_tensor(pos).cuda()
    md = torch.as_tensor(m).cuda()
    lines = []
    for theta in thetas:
        leaf, times = precision.autotune_leaf_size(pd, md, theta=theta, softening=eps, G=G,
                                                   form="fp32", criterion=criterion)
        _log(f"theta={theta}: autotune {times}")
        t32 = api.Tree(pd, md, leaf_size=leaf, form="fp32", criterion=criterion).build()
        a32, s32 = _timed_solve(t32, theta, eps, G)
        p2p, m2p, _ = t32._handle.stats()
        t32.close()
        t64 = api.Tree(pd, md, leaf_size=leaf, form="fast").build()
        _log(f"theta={theta}: fp32 solve {s32:.3f} s")
        a64, s64 = _timed_solve(t64, theta, eps, G, reps=1)
        fb = t64._handle.fallbacks()
        t64.close()
        _log(f"theta={theta}: fast solve {s64:.3f} s")
        a32h = a32.cpu().numpy()
        a64h = a64.cpu().numpy()
        line = {
            "report": "precision", "workload": f"galaxy N={n:,} (70% exponential disc Rd=3, "
            "z0=0.3; 30% Hernquist bulge a=0.5; equal masses)", "theta": theta,
            "softening": eps, "criterion": criterion, "leaf_size": leaf,
            "autotune_s": {str(k): v for k, v in times.items()},
            "fp32": {"accels_per_s": n / s32, "solve_ms": 1e3 * s32,
                     "err_vs_direct": precision.error_distribution(a32h[idx], ref),
                     "err_vs_fp64_plain": precision.error_distribution(a32h, a64h)},
            "fp64_fast": {"accels_per_s": n / s64, "solve_ms": 1e3 * s64,
                          "fp64_fallback_decisions": fb[0], "fp64_pairs": fb[1],
                          "err_vs_direct": precision.error_distribution(a64h[idx], ref)},
            "interactions": {"p2p": p2p, "m2p": m2p},
            "direct_sum": {"targets": len(idx), "seconds": t_direct},
        }
        print(json.dumps(line), flush=True)
        lines.append(line)
    return lines


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("report", choices=["precision"])
    ap.add_argument("--n", type=int, default=4_000_000)
    ap.add_argument("--sample", type=int, default=8192)
    ap.add_argument("--criterion", default="bh")
    ap.add_argument("--thetas", default="0.3,0.5,0.7")
    args = ap.parse_args()
    if args.report == "precision":
        precision_report(args.n, args.sample, criterion=args.criterion,
                         thetas=tuple(float(x) for x in args.thetas.split(",")))


if __name__ == "__main__":
    main()
