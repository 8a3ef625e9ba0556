"""Measurement reports for the engine's forms beyond the plain FP64 path.

    python -m bhut_gb300.reports precision [--n 4000000] [--sample 8192]
    python -m bhut_gb300.reports batched [--nsys 2048]
    python -m bhut_gb300.reports served [--count 24] [--theta 0.7]
    python -m bhut_gb300.reports scaling [--sizes 1e5,1e6,4e6,16e6,64e6]
    python -m bhut_gb300.reports build [--n 1000000] [--reps 10]

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
                     eps: float = 0.005, G: float = 1.0, seed: int = 7, criterion: str = "bh",
                     multipole: str = "mono"):
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
                                                   form="fp32", criterion=criterion,
                                                   multipole=multipole)
        _log(f"theta={theta}: autotune {times}")
        t32 = api.Tree(pd, md, leaf_size=leaf, form="fp32", criterion=criterion,
                       multipole=multipole).build()
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
            "softening": eps, "criterion": criterion, "multipole": multipole, "leaf_size": leaf,
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


def batched_report(nsys: int = 2048, nmin: int = 256, nmax: int = 65536, seed: int = 11,
                   theta: float = 0.5, eps: float = 0.01, G: float = 1.0, reps: int = 3,
                   plain_sample: int = 64, err_systems: int = 16, criterion: str = "bh",
                   multipole: str = "mono"):
    """``batched``: nsys Plummer spheres (N log-uniform in [nmin, nmax], scale
    radius uniform in [0.5, 2], own seeds, equal masses 1/N) solved in one
    batch (FP32 form, CUDA graph, autotuned leaf size and targets per warp);
    systems/s and accels/s, against the plain per-system GPU path (one
    single-tree FP64-accurate solve per system) timed on a sample of the
    systems; errors vs FP64 direct sum on sampled systems."""
    import torch
    from . import batch
    systems = workloads.plummer_batch(nsys, nmin, nmax, seed=seed)
    pos, m, off = batch.concat_systems(systems)
    ntot = int(off[-1])
    _log(f"{nsys} systems, {ntot:,} particles")
    pd = torch.as_tensor(pos).cuda()
    md = torch.as_tensor(m).cuda()
    cfg, times = batch.autotune(pd, md, off, theta=theta, softening=eps, G=G, form="fp32",
                                criterion=criterion, multipole=multipole)
    _log(f"autotune {cfg} {times}")
    sv = batch.BatchedSolver(leaf_size=cfg["leaf_size"], form="fp32", criterion=criterion,
                             targets_per_warp=cfg["targets_per_warp"], use_graph=True,
                             multipole=multipole, stack=cfg["stack"])
    sv.load(pd, md, off)
    out = torch.empty_like(pd)
    sv.solve(theta=theta, softening=eps, G=G, out=out)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(reps):
        sv.solve(theta=theta, softening=eps, G=G, out=out)
    ev1.record()
    ev1.synchronize()
    t_batch = ev0.elapsed_time(ev1) / 1e3 / reps
    p2p, m2p, _ = sv.stats()
    acc = out.cpu().numpy()
    sv.close()
    _log(f"batched solve {t_batch * 1e3:.2f} ms")
    # plain per-system GPU path (form fast, one Tree per system) on a sample
    rng = np.random.default_rng(seed + 1)
    pick = rng.choice(nsys, min(plain_sample, nsys), replace=False)
    t_plain = 0.0
    n_plain = 0
    for s in pick:
        p_, m_ = systems[s]
        tr = api.Tree(p_, m_, leaf_size=32, form="fast").build()
        tr.accelerations(theta=theta, softening=eps, G=G)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr.rebuild(p_, m_)
        tr.accelerations(theta=theta, softening=eps, G=G)
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t0
        n_plain += len(m_)
        tr.close()
    plain_sps = len(pick) / t_plain
    _log(f"plain path: {len(pick)} systems in {t_plain:.3f} s")
    # accuracy on sampled systems vs FP64 direct sum (all their particles)
    errs, pooled, sizes = [], [], []
    for s in rng.choice(nsys, min(err_systems, nsys), replace=False):
        p_, m_ = systems[s]
        ref = np.asarray(api.direct_accelerations(p_, m_, softening=eps, G=G))
        a_ = acc[off[s]:off[s + 1]]
        errs.append(precision.error_distribution(a_, ref))
        sizes.append(len(m_))
        den = np.linalg.norm(ref, axis=1)
        pooled.append(np.linalg.norm(a_ - ref, axis=1)[den > 0] / den[den > 0])
    pooled = np.concatenate(pooled)
    line = {
        "report": "batched", "workload": f"{nsys} Plummer spheres, N log-uniform in "
        f"[{nmin}, {nmax}], a ~ U[0.5, 2], own seeds", "particles": ntot, "theta": theta,
        "softening": eps, "form": "fp32", "criterion": criterion, "multipole": multipole,
        "config": cfg,
        "autotune_s": {f"L{k[0]}_tpw{k[1]}_{k[2]}": v for k, v in times.items()},
        "solve_ms": t_batch * 1e3, "systems_per_s": nsys / t_batch,
        "accels_per_s": ntot / t_batch, "interactions": {"p2p": p2p, "m2p": m2p},
        "plain_per_system": {"systems_timed": int(len(pick)), "systems_per_s": plain_sps,
                             "particles": n_plain, "seconds": t_plain},
        "speedup_systems_per_s": (nsys / t_batch) / plain_sps,
        "err_vs_direct_median_of_medians": float(np.median([e["median"] for e in errs])),
        "err_vs_direct_worst_p99": float(max(e["p99"] for e in errs)),
    }
    print(json.dumps(line), flush=True)
    return line


def served_report(count: int = 24, rate: float = 200.0, steps: int = 100, seed: int = 21,
                  plain_seconds: float = 90.0, err_requests: int = 6, theta: float = 0.7,
                  criterion: str = "bh_offset", multipole: str = "quad",
                  plain_theta: float = 0.5, closed_loop: bool = True, emit: bool = True,
                  plain_theta_equal_error: float | None = None):
    """``served``: a Poisson stream (mean ``rate`` requests/s) of ``count``
    systems (N log-uniform in [1e3, 2e6], half Plummer, half uniform cubes of
    side 2, velocities N(0, 0.1^2)), each advanced ``steps`` KDK steps
    (dt = 1e-3, eps = 0.01), refit every step, rebuild every 10; the
    continuous-batching server (FP32 form; by default theta 0.7, offset
    criterion, quadrupoles) against the plain per-request path (form fast,
    the reference's monopole/theta 0.5 configuration), both in real time from
    the same arrival schedule; latencies include queueing.  With
    ``closed_loop`` the server also runs the stream saturated (every request
    queued at t = 0).  Median errors vs FP64 direct sum on the initial
    conditions of requests spread over the size range, for both
    configurations.  ``plain_theta_equal_error`` adds a second plain run at
    a smaller theta whose error is close to the server's (equal-error
    comparison)."""
    from . import serve
    reqs = serve.request_stream(count, rate=rate, steps=steps, seed=seed)
    total_n = sum(r.n for r in reqs)
    _log(f"{count} requests, {total_n:,} particles")
    errs_srv, errs_plain, errs_eq = [], [], []
    by_size = sorted(reqs, key=lambda r: r.n)
    pick = [by_size[int(round(k))] for k in np.linspace(0, len(by_size) - 1, err_requests)]
    for r in pick:
        idx = precision.sample_indices(r.n, 2048, seed=1)
        ref = precision.direct_reference(r.positions, r.masses, idx, softening=0.01)
        a_s = api.accelerations(r.positions, r.masses, theta=theta, softening=0.01,
                                form="fp32", criterion=criterion, multipole=multipole,
                                leaf_size=16)
        a_p = api.accelerations(r.positions, r.masses, theta=plain_theta, softening=0.01,
                                form="fast")
        errs_srv.append(precision.error_distribution(a_s[idx], ref)["median"])
        errs_plain.append(precision.error_distribution(a_p[idx], ref)["median"])
        if plain_theta_equal_error is not None:
            a_q = api.accelerations(r.positions, r.masses, theta=plain_theta_equal_error,
                                    softening=0.01, form="fast")
            errs_eq.append(precision.error_distribution(a_q[idx], ref)["median"])
    _log(f"median errors: served {errs_srv}, plain {errs_plain}")
    # warm-up: two small requests through a throwaway server load the batched
    # kernels and grow the memory pools (the plain path's kernels were loaded
    # by the error measurement above)
    wp, wm = workloads.plummer(4096, seed=5)
    warm = [serve.Request(-1 - k, 0.0, wp, np.zeros_like(wp), wm, steps=12) for k in range(2)]
    sv = serve.Server(theta=theta, softening=0.01, dt=1e-3, rebuild_every=10, form="fp32",
                      criterion=criterion, multipole=multipole)
    sv.run(warm, realtime=False)
    sv.close()
    sv = serve.Server(theta=theta, softening=0.01, dt=1e-3, rebuild_every=10, form="fp32",
                      criterion=criterion, multipole=multipole)
    st = sv.run(reqs, realtime=True)
    sv.close()
    _log(f"served: {st}")
    closed = None
    if closed_loop:
        sv = serve.Server(theta=theta, softening=0.01, dt=1e-3, rebuild_every=10, form="fp32",
                          criterion=criterion, multipole=multipole)
        closed = sv.run(serve.request_stream(count, rate=rate, steps=steps, seed=seed),
                        realtime=False)
        sv.close()
        _log(f"served, closed loop: {closed}")
    reqs2 = serve.request_stream(count, rate=rate, steps=steps, seed=seed)
    pl = serve.plain_path(reqs2, theta=plain_theta, softening=0.01, dt=1e-3, rebuild_every=10,
                          realtime=True, max_seconds=plain_seconds)
    _log(f"plain: {pl}")
    equal = None
    if plain_theta_equal_error is not None:
        th2 = plain_theta_equal_error
        e2 = errs_eq
        pl2 = serve.plain_path(serve.request_stream(count, rate=rate, steps=steps, seed=seed),
                               theta=th2, softening=0.01, dt=1e-3, rebuild_every=10,
                               realtime=True, max_seconds=plain_seconds)
        equal = {"theta": th2, "plain": pl2, "median_err_vs_direct": float(np.median(e2)),
                 "solves_per_s_ratio": st["solves_per_s"] / pl2["solves_per_s"]
                 if pl2["solves_per_s"] else None}
        _log(f"plain at theta={th2}: {equal}")
    line = {"report": "served", "requests": count, "rate_per_s": rate, "steps": steps,
            "particles": total_n,
            "served_config": {"form": "fp32", "theta": theta, "criterion": criterion,
                              "multipole": multipole, "leaf_size": 16},
            "plain_config": {"form": "fast", "theta": plain_theta, "criterion": "bh",
                             "multipole": "mono", "leaf_size": 32},
            "served": st, "served_closed_loop": closed, "plain": pl,
            "plain_equal_error": equal,
            "solves_per_s_ratio": st["solves_per_s"] / pl["solves_per_s"]
            if pl["solves_per_s"] else None,
            "err_requests_n": [r.n for r in pick],
            "median_err_vs_direct": {"served": float(np.median(errs_srv)),
                                     "plain": float(np.median(errs_plain)),
                                     "served_per_request": errs_srv,
                                     "plain_per_request": errs_plain}}
    if emit:
        print(json.dumps(line), flush=True)
    return line


def scaling_report(sizes=(100_000, 1_000_000, 4_000_000, 16_000_000, 64_000_000),
                   forms=("fast", "fp32"), theta: float = 0.5, eps: float = 0.01, reps: int = 2):
    """``scaling``: self accelerations of Plummer spheres of growing N
    (theta 0.5, eps 0.01, leaf 32), build and traversal timed separately
    through one persistent tree handle; accels/s and interactions per
    target for each form."""
    import torch
    from .api import _Handle
    lines = []
    for n in sizes:
        pos, m = workloads.plummer(int(n), seed=3)
        pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
        out = torch.empty_like(pd)
        for form in forms:
            h = _Handle(3, 32)
            h.set_form(form)
            best_b = best_t = float("inf")
            for r in range(reps + 1):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                h.build(pd, md)
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                h.accel_self(theta, eps, 1.0, out)
                torch.cuda.synchronize()
                t2 = time.perf_counter()
                if r:
                    best_b, best_t = min(best_b, t1 - t0), min(best_t, t2 - t1)
            p2p, m2p, visits = h.stats()
            h.close()
            line = {"report": "scaling", "n": int(n), "form": form, "theta": theta,
                    "build_ms": best_b * 1e3, "traversal_ms": best_t * 1e3,
                    "accels_per_s": n / (best_b + best_t),
                    "p2p_per_target": p2p / n, "m2p_per_target": m2p / n,
                    "visits_per_target": visits / n}
            _log(f"N={n:,} {form}: {line['accels_per_s']:.3g} accels/s")
            print(json.dumps(line), flush=True)
            lines.append(line)
        del pd, md, out
    return lines


def build_report(n: int = 1_000_000, reps: int = 10, leaf: int = 32, seed: int = 1):
    """``build``: rebuilds of a Plummer sphere of n particles through one
    persistent tree handle (staging copy + bounding box, Morton keys, radix
    sort, gather, bottom-up moments: bhut.Tree.rebuild), then as many refits
    in place (bottom-up moments only), the inputs resident on the device.
    Each call is timed with CUDA events on the handle's stream; one JSON line
    with the medians and the minima."""
    import torch
    from .api import _Handle
    pos, m = workloads.plummer(int(n), seed=seed)
    pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
    stream = torch.cuda.Stream()
    h = _Handle(3, leaf, stream=stream.cuda_stream)
    h.build(pd, md)
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.rebuild(pd, md)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    refits = []   # refit in place (same topology: bhut.Tree.refit), positions moved
    moved = pd + 1e-3 * torch.randn_like(pd)
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.refit_only(moved, md)
        e1.record(stream)
        e1.synchronize()
        refits.append(e0.elapsed_time(e1))
    h.close()
    times.sort()
    refits.sort()
    line = {"report": "build", "n": int(n), "leaf_size": leaf, "reps": reps,
            "rebuild_ms_median": times[len(times) // 2], "rebuild_ms_min": times[0],
            "refit_ms_median": refits[len(refits) // 2], "refit_ms_min": refits[0]}
    print(json.dumps(line), flush=True)
    return line


# ---------------------------------------------------------------------------
# Sub-records of the benchmark line (bench.py): each bounded in time
# ---------------------------------------------------------------------------
# FP32-pipe operations per evaluation, counted from bhut_gb300/csrc/fast.cuh:
# a pair term into a leaf partial (pair_f32_partial2: displacement 9,
# r^2 + eps^2 3, cube 2, m * w 1 -- none in the unit-mass frame -- three
# FMAs 3; the x and y operations run as f32x2 instructions, two operations
# per issue), a Kahan-added monopole (pair_f32: the same 15 plus a Kahan step
# per component 12), a Kahan-added monopole + quadrupole node (node_quad_f32:
# displacement 9, r^2 3, powers 3, Q d 9, d.Q d 3, force factor 4, per
# component 6 -> 49), each plus one MUFU rsqrt.  Every workload here has
# equal masses (the unit-mass frame).
F32_OPS_PER_PAIR = 17
F32_OPS_PER_MONOPOLE = 27
F32_OPS_PER_QUAD_NODE = 49


def fp32_ops(p2p: int, m2p: int, multipole: str) -> int:
    node = F32_OPS_PER_QUAD_NODE if multipole == "quad" else F32_OPS_PER_MONOPOLE
    return F32_OPS_PER_PAIR * p2p + node * m2p


def fp32_roofline(ops: int, seconds: float, fma_rate: float, kernel: str, multipole: str) -> dict:
    """Achieved FP32-pipe operations per second of a traversal against the
    FP32 FMA lane rate measured in the same run (T ops/s)."""
    achieved = ops / seconds / 1e12
    node = F32_OPS_PER_QUAD_NODE if multipole == "quad" else F32_OPS_PER_MONOPOLE
    return {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": fma_rate,
            "unit": "T FP32-pipe ops/s", "frac": achieved / fma_rate,
            "work_per_launch": int(ops),
            "work_rule": f"{F32_OPS_PER_PAIR} FP32 ops per pair term (unit-mass frame), {node} "
                         f"per {'monopole+quadrupole' if multipole == 'quad' else 'monopole'} "
                         "node, x evaluations counted by the kernel",
            "peak_source": "independent FP32 FMA chains on every SM, measured in this run"}


def exact_record(pos_d, m_d, *, theta: float, eps: float, G: float, leaf: int,
                 fp64_peak: float) -> dict:
    """The IEEE-FP64 form (form "exact") at the headline workload: one
    rebuild + traversal, device time by CUDA events on the handle's stream."""
    import torch
    from .api import _Handle
    n = int(pos_d.shape[0])
    stream = torch.cuda.Stream()
    h = _Handle(3, leaf, stream=stream.cuda_stream)
    h.set_form("exact")
    out = torch.empty_like(pos_d)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    h.rebuild(pos_d, m_d)
    e1.record(stream)
    h.accel_self(theta, eps, G, out)
    e2.record(stream)
    e2.synchronize()
    trav = e1.elapsed_time(e2) / 1e3
    total = e0.elapsed_time(e2) / 1e3
    p2p, m2p, visits = h.stats()
    h.close()
    flops = 20 * (p2p + m2p)
    achieved = flops / trav / 1e12
    return {"form": "exact", "arith": "IEEE FP64", "dtype": "f64", "accels_per_s": n / total,
            "solve_ms": total * 1e3, "traversal_ms": trav * 1e3,
            "roofline": {"bound": "fp64", "kernel": "k_traverse_exact", "achieved": achieved,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                         "work_rule": "20 flop x (pair + monopole evaluations counted by the "
                                      "kernel)",
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"},
            "interactions_per_solve": {"p2p": p2p, "m2p": m2p, "node_visits": visits}}


def c2_sequence_record(pos_d, m_d, *, theta: float, eps: float, G: float, leaf: int,
                       n_targets: int = 250_000, reps: int = 3) -> dict:
    """The rest of the 1M Plummer sequence, form "fast", through one tree
    handle (bhut.Tree): accelerations at external targets uniform in a
    centred cube of side 10, then a refit after positions += 0.01 N(0, 1)
    (bhut/tree/refit.py: refit, or a rebuild when a particle left 1.1x the
    root box) followed by a self solve, then a rebuild of the moved particles
    followed by a self solve.  Each step's device time by CUDA events on the
    handle's stream, median of ``reps``, inputs resident on the device."""
    import torch
    from .api import _Handle
    n = int(pos_d.shape[0])
    tg = torch.as_tensor(workloads.cube_targets(n_targets, seed=5, side=10.0)).cuda()
    gen = torch.Generator(device="cuda").manual_seed(6)
    moved = pos_d + 0.01 * torch.randn(pos_d.shape, dtype=pos_d.dtype, device="cuda",
                                       generator=gen)
    stream = torch.cuda.Stream()
    h = _Handle(3, leaf, stream=stream.cuda_stream)
    h.set_form("fast")
    out_t = torch.empty((n_targets, 3), dtype=torch.float64, device="cuda")
    out = torch.empty_like(pos_d)

    def timed(fn):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        ts.sort()
        return ts[len(ts) // 2], r

    h.build(pos_d, m_d)
    h.accel_targets(tg, theta, eps, G, out_t)          # first call: target buffers
    t_tg, _ = timed(lambda: h.accel_targets(tg, theta, eps, G, out_t))
    p2p_t, m2p_t, _ = h.stats()
    # refit of the built tree to the moved positions (repeating it with the
    # same positions leaves the same tree), then its solve
    t_r, rebuilt = timed(lambda: h.refit(moved, m_d))
    t_rs, _ = timed(lambda: h.accel_self(theta, eps, G, out))
    t_rb, _ = timed(lambda: h.rebuild(moved, m_d))
    t_rbs, _ = timed(lambda: h.accel_self(theta, eps, G, out))
    h.close()
    return {"workload": f"Plummer N={n:,} (seed 1), form fast: {n_targets:,} external targets "
                        "uniform in [-5, 5]^3 (seed 5), refit after positions += 0.01 N(0,1) "
                        "(seed 6), rebuild",
            "targets": {"accels_per_s": n_targets / t_tg, "ms": t_tg * 1e3,
                        "interactions": {"p2p": p2p_t, "m2p": m2p_t}},
            "refit": {"ms": t_r * 1e3, "fell_back_to_rebuild": bool(rebuilt),
                      "solve_ms": t_rs * 1e3},
            "rebuild": {"ms": t_rb * 1e3, "solve_ms": t_rbs * 1e3},
            "note": "refit and rebuild ms include the input check and error-word round trips "
                    "to the host; medians of " + str(reps)}


def c1_record(*, n: int = 10_000, theta: float = 0.5, eps: float = 0.01, G: float = 1.0,
              leaf: int = 32, steps: int = 50, e2e_calls: int = 20,
              fma_rate: float | None = None):
    """The reference's CPU-runnable workload: n Gaussian particles (seed 0,
    unit masses), theta 0.5, softening 0.01, leaf 32, self accelerations,
    form "fast".  Device time of rebuild + traversal through one persistent
    handle (CUDA events, median of ``steps``), and end to end through
    bhut_gb300.accelerations with host NumPy buffers.  Returns the record
    and the accelerations (for the caller's CPU comparison)."""
    import torch
    from .api import _Handle
    pos, m = workloads.gaussian(n, seed=0)
    pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
    out = torch.empty_like(pd)
    stream = torch.cuda.Stream()
    h = _Handle(3, leaf, stream=stream.cuda_stream)
    h.set_form("fast")
    h.build(pd, md)
    h.accel_self(theta, eps, G, out)
    torch.cuda.synchronize()
    tot, trav = [], []
    for _ in range(steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        h.rebuild(pd, md)
        e1.record(stream)
        h.accel_self(theta, eps, G, out)
        e2.record(stream)
        e2.synchronize()
        tot.append(e0.elapsed_time(e2) / 1e3)
        trav.append(e1.elapsed_time(e2) / 1e3)
    p2p, m2p, visits = h.stats()
    h.close()
    tot.sort()
    trav.sort()
    t_step, t_trav = tot[len(tot) // 2], trav[len(trav) // 2]
    api.accelerations(pos, m, theta=theta, softening=eps, G=G, leaf_size=leaf)
    t0 = time.perf_counter()
    for _ in range(e2e_calls):
        acc = api.accelerations(pos, m, theta=theta, softening=eps, G=G, leaf_size=leaf)
    t_e2e = (time.perf_counter() - t0) / e2e_calls
    rec = {"workload": f"Gaussian N={n:,} (standard normal positions, seed 0, unit masses), "
                       f"theta={theta}, softening={eps}, G={G}, leaf_size={leaf}, self "
                       "accelerations, form fast",
           "accels_per_s": n / t_step, "solve_ms_median": t_step * 1e3,
           "traversal_ms_median": t_trav * 1e3, "steps": steps,
           "e2e": {"value": n / t_e2e, "unit": "accels/s", "api": "bhut_gb300.accelerations",
                   "timed_calls": e2e_calls, "h2d_bytes_per_call": int(pos.nbytes + m.nbytes),
                   "d2h_bytes_per_call": int(acc.nbytes)},
           "interactions_per_solve": {"p2p": p2p, "m2p": m2p, "node_visits": visits}}
    if fma_rate:
        instr = 93 * p2p + 97 * m2p
        rec["roofline"] = {"bound": "fp32", "kernel": "k_traverse_fast",
                           "achieved": instr / t_trav / 1e12, "peak": fma_rate,
                           "unit": "T instr/s", "frac": instr / t_trav / 1e12 / fma_rate,
                           "note": "10,000 targets at 4 lanes each (k_traverse_fast_lpt) are "
                                   "1,250 warps for 152 SMs: latency-bound at this size (the "
                                   "traversal time includes the launch)"}
    return rec, np.asarray(acc), (pos, m)


def batched_record(*, nsys: int = 2048, nmin: int = 256, nmax: int = 65536, seed: int = 11,
                   theta: float = 0.5, eps: float = 0.01, G: float = 1.0,
                   multipole: str = "quad", reps: int = 3, plain_sample: int = 64,
                   err_systems: int = 16, fma_rate: float | None = None) -> dict:
    """The batched form on its named workload: ``nsys`` Plummer spheres in one
    CUDA-graph solve (FP32 form, autotuned leaf / targets per warp / stack),
    systems/s and accels/s, error against FP64 direct sums, the plain
    per-system path on a sample, and the roofline of k_batch_traverse."""
    import torch
    from . import batch
    systems = workloads.plummer_batch(nsys, nmin, nmax, seed=seed)
    pos, m, off = batch.concat_systems(systems)
    ntot = int(off[-1])
    pd = torch.as_tensor(pos).cuda()
    md = torch.as_tensor(m).cuda()
    t0 = time.perf_counter()
    cfg, times = batch.autotune(pd, md, off, theta=theta, softening=eps, G=G, form="fp32",
                                multipole=multipole, repeats=1)
    t_tune = time.perf_counter() - t0
    sv = batch.BatchedSolver(leaf_size=cfg["leaf_size"], form="fp32",
                             targets_per_warp=cfg["targets_per_warp"], use_graph=True,
                             multipole=multipole, stack=cfg["stack"])
    sv.load(pd, md, off)
    out = torch.empty_like(pd)
    sv.solve(theta=theta, softening=eps, G=G, out=out)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    trav = []
    ev0.record()
    for _ in range(reps):
        sv.solve(theta=theta, softening=eps, G=G, out=out)
        trav.append(sv.traverse_ms() / 1e3)
    ev1.record()
    ev1.synchronize()
    t_batch = ev0.elapsed_time(ev1) / 1e3 / reps
    p2p, m2p, _ = sv.stats()
    acc = out.cpu().numpy()
    sv.close()
    rng = np.random.default_rng(seed + 1)
    pick = rng.choice(nsys, min(plain_sample, nsys), replace=False)
    t_plain = 0.0
    for s in pick:
        p_, m_ = systems[s]
        tr = api.Tree(p_, m_, leaf_size=32, form="fast").build()
        tr.accelerations(theta=theta, softening=eps, G=G)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        tr.rebuild(p_, m_)
        tr.accelerations(theta=theta, softening=eps, G=G)
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t1
        tr.close()
    plain_sps = len(pick) / t_plain
    errs, pooled, sizes = [], [], []
    for s in rng.choice(nsys, min(err_systems, nsys), replace=False):
        p_, m_ = systems[s]
        ref = np.asarray(api.direct_accelerations(p_, m_, softening=eps, G=G))
        a_ = acc[off[s]:off[s + 1]]
        errs.append(precision.error_distribution(a_, ref))
        sizes.append(len(m_))
        den = np.linalg.norm(ref, axis=1)
        pooled.append(np.linalg.norm(a_ - ref, axis=1)[den > 0] / den[den > 0])
    pooled = np.concatenate(pooled)
    t_trav = float(np.median(trav))
    rec = {
        "workload": f"{nsys} Plummer spheres, N log-uniform in [{nmin}, {nmax}] "
                    f"({ntot:,} particles), a ~ U[0.5, 2], own seeds, equal masses 1/N",
        "theta": theta, "softening": eps, "form": "fp32", "arith": "FP32 + Kahan; FP64 keys, "
        "centres of mass and quadrupoles", "criterion": "bh", "multipole": multipole,
        "config": cfg, "autotune_s": t_tune, "cuda_graph": True,
        "solve_ms": t_batch * 1e3, "traversal_ms": t_trav * 1e3,
        "systems_per_s": nsys / t_batch, "accels_per_s": ntot / t_batch,
        "interactions": {"p2p": p2p, "m2p": m2p},
        "plain_per_system": {"form": "fast", "systems_timed": int(len(pick)),
                             "systems_per_s": plain_sps},
        "speedup_vs_plain_systems_per_s": (nsys / t_batch) / plain_sps,
        "err_vs_fp64_direct": {"systems": len(errs),
                               "median_over_particles": float(np.median(pooled)),
                               "p99_over_particles": float(np.percentile(pooled, 99)),
                               "median_of_medians": float(np.median([e["median"] for e in errs])),
                               "worst_p99": float(max(e["p99"] for e in errs)),
                               "median_by_system": [[int(n_), e["median"]] for n_, e in
                                                    sorted(zip(sizes, errs),
                                                           key=lambda x: x[0])],
                               "note": "systems small enough that every leaf is opened are "
                                       "summed directly (error at FP32 rounding), so the "
                                       "median of medians is low; the pooled figures weight "
                                       "each system by its particles"},
    }
    if fma_rate:
        rec["roofline"] = fp32_roofline(fp32_ops(p2p, m2p, multipole), t_trav, fma_rate,
                                        "k_batch_traverse", multipole)
    return rec


def precision_record(*, n: int = 4_000_000, n_sample: int = 8192, thetas=(0.3, 0.5, 0.7),
                     eps: float = 0.005, G: float = 1.0, seed: int = 7,
                     fma_rate: float | None = None) -> dict:
    """The precision form on its named workload (galaxy disc + bulge):
    per theta an autotuned leaf size, FP32/Kahan accels/s with the roofline of
    k_traverse_fp32, its error distribution against the FP64 direct sum on
    sampled targets and against the FP64-accurate form on all targets."""
    import torch
    from .api import _Handle
    pos, m = workloads.galaxy(n, seed=seed)
    idx = precision.sample_indices(n, n_sample, seed=seed + 1)
    ref = precision.direct_reference(pos, m, idx, softening=eps, G=G)
    pd = torch.as_tensor(pos).cuda()
    md = torch.as_tensor(m).cuda()
    out = torch.empty_like(pd)
    stream = torch.cuda.Stream()
    rows = []
    for theta in thetas:
        leaf, times = precision.autotune_leaf_size(pd, md, theta=theta, softening=eps, G=G,
                                                   form="fp32", repeats=1)
        h = _Handle(3, leaf, stream=stream.cuda_stream)
        h.set_form("fp32")
        h.rebuild(pd, md)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        h.rebuild(pd, md)
        e1.record(stream)
        h.accel_self(theta, eps, G, out)
        e2.record(stream)
        e2.synchronize()
        trav = e1.elapsed_time(e2) / 1e3
        total = e0.elapsed_time(e2) / 1e3
        p2p, m2p, _ = h.stats()
        a32 = out.cpu().numpy()
        h.set_form("fast")
        h.accel_self(theta, eps, G, out)
        a64 = out.cpu().numpy()
        h.close()
        row = {"theta": theta, "leaf_size": leaf,
               "autotune_s": {str(k): v for k, v in times.items()},
               "accels_per_s": n / total, "solve_ms": total * 1e3, "traversal_ms": trav * 1e3,
               "err_vs_fp64_direct": precision.error_distribution(a32[idx], ref),
               "err_vs_fp64_form_fast": precision.error_distribution(a32, a64),
               "fast_err_vs_fp64_direct": precision.error_distribution(a64[idx], ref),
               "interactions": {"p2p": p2p, "m2p": m2p}}
        if fma_rate:
            row["roofline"] = fp32_roofline(fp32_ops(p2p, m2p, "mono"), trav, fma_rate,
                                            "k_traverse_fp32", "mono")
        rows.append(row)
    return {"workload": f"galaxy N={n:,}: 70% exponential disc (Rd 3.0, sech^2 z0 0.3), 30% "
                        "Hernquist bulge (a 0.5), equal masses", "softening": eps,
            "form": "fp32", "arith": "FP32 + Kahan; FP64 bbox, keys and centres of mass",
            "multipole": "mono", "sampled_targets": int(len(idx)), "by_theta": rows}


def served_record(*, count: int = 200, rate: float = 200.0, steps: int = 100, seed: int = 21,
                  server_seconds: float = 45.0, full_steps: int = 10, sample_requests: int = 40,
                  solve_budget: int = 1_000_000, theta: float = 0.7,
                  criterion: str = "bh_offset", multipole: str = "quad", leaf: int = 16,
                  fast_theta: float = 0.33, err_requests: int = 6,
                  hbm_budget: float = 150e9) -> dict:
    """The served form on its named stream (Poisson ``rate``/s, N log-uniform
    in [1e3, 2e6], half Plummer half cubes, ``steps`` KDK steps, refit every
    step, rebuild every 10, HBM budget 150 GB) against the plain per-request
    path, in two comparisons:

    * stream: the server runs the open-loop stream in real time for
      ``server_seconds`` (latency p50/p99 by size class, solves done in the
      window).  The plain path (one request at a time, shortest work first
      among the arrived ones, as the server) is scheduled on the same stream
      and window from its measured per-request costs.
    * full stream: every request advanced ``full_steps`` steps (a rebuild
      at the 10th), all queued at t=0: the server's makespan, measured,
      against the plain path's sum of per-request costs.  In both, solves/s
      counts every request-step once, whatever its size.

    The plain path's cost of a request (initial solve, refit step, rebuild
    step; ``serve.plain_service_times``) is measured on ``sample_requests``
    requests spread over the size range and interpolated in N for the
    others (leave-one-out error reported).  Two plain configurations: the
    server's own (form fp32, theta, criterion, multipole, leaf: the same
    arithmetic per system, equal error by construction -- the ratio isolates
    batching and residency) and the FP64-accurate form ``fast`` with the
    reference's criterion at a theta whose error against FP64 direct sums
    is close to the server's."""
    import dataclasses
    from . import serve
    base = serve.request_stream(count, rate=rate, steps=steps, seed=seed)
    fresh = lambda k=steps: [dataclasses.replace(r, steps=k) for r in base]  # noqa: E731
    total_n = sum(r.n for r in base)
    by_size = sorted(base, key=lambda r: r.n)
    pick = [by_size[int(round(k))] for k in np.linspace(0, len(by_size) - 1, err_requests)]
    e_srv, e_fast, e_fast05 = [], [], []
    for r in pick:
        idx = precision.sample_indices(r.n, 2048, seed=1)
        ref = precision.direct_reference(r.positions, r.masses, idx, softening=0.01)
        a_s = api.accelerations(r.positions, r.masses, theta=theta, softening=0.01, form="fp32",
                                criterion=criterion, multipole=multipole, leaf_size=leaf)
        a_f = api.accelerations(r.positions, r.masses, theta=fast_theta, softening=0.01,
                                form="fast")
        a_5 = api.accelerations(r.positions, r.masses, theta=0.5, softening=0.01, form="fast")
        e_srv.append(precision.error_distribution(a_s[idx], ref)["median"])
        e_fast.append(precision.error_distribution(a_f[idx], ref)["median"])
        e_fast05.append(precision.error_distribution(a_5[idx], ref)["median"])
    kw = dict(theta=theta, softening=0.01, dt=1e-3, rebuild_every=10, form="fp32",
              criterion=criterion, multipole=multipole, leaf_size=leaf)
    wp, wm = workloads.plummer(4096, seed=5)
    warm = [serve.Request(-1 - k, 0.0, wp, np.zeros_like(wp), wm, steps=12) for k in range(2)]
    sv = serve.Server(**kw)
    sv.run(warm, realtime=False)
    sv.close()
    sv = serve.Server(**kw, hbm_budget=hbm_budget, solve_budget=solve_budget)
    st = sv.run(fresh(), realtime=True, max_seconds=server_seconds)
    sv.close()
    sv = serve.Server(**kw, hbm_budget=hbm_budget, solve_budget=solve_budget)
    full = sv.run(fresh(full_steps), realtime=False)
    sv.close()
    full_server = {"solves": full["solves"], "wall_s": full["wall_s"],
                   "solves_per_s": full["solves_per_s"], "accels_per_s": full["accels_per_s"],
                   "requests_done": full["requests_done"]}

    spread = [by_size[int(round(k))] for k in np.linspace(0, len(by_size) - 1,
                                                          min(sample_requests, count))]
    plain_cfgs = {
        "plain_same_config": dict(theta=theta, form="fp32", criterion=criterion,
                                  multipole=multipole, leaf_size=leaf),
        "plain_fast_equal_error": dict(theta=fast_theta, form="fast", criterion="bh",
                                       multipole="mono", leaf_size=32),
    }
    plain = {}
    for name, cfg in plain_cfgs.items():
        t0 = time.perf_counter()
        meas = serve.plain_service_times(spread, softening=0.01, dt=1e-3, **cfg)
        t_meas = time.perf_counter() - t0
        costs = serve.interpolate_service_times(meas, base)
        loo = []   # leave-one-out: each measured request predicted from the others
        for k, t in enumerate(meas):
            rest = meas[:k] + meas[k + 1:]
            r = next(q for q in base if q.rid == t["rid"])
            est = serve.interpolate_service_times(rest, [r])[r.rid]
            c_true = serve.request_cost(t, steps, 10)
            loo.append(abs(serve.request_cost(est, steps, 10) - c_true) / c_true)
        full_s = sum(serve.request_cost(costs[r.rid], full_steps, 10) for r in base)
        window = serve.simulate_sequential(base, costs, steps=steps, rebuild_every=10,
                                           order="shortest", window=server_seconds)
        whole = serve.simulate_sequential(base, costs, steps=steps, rebuild_every=10,
                                          order="shortest")
        plain[name] = {
            "config": cfg,
            "stream_window": window,
            "stream_to_completion": {k: whole[k] for k in ("wall_s", "solves_per_s",
                                                           "latency_p50_s", "latency_p99_s",
                                                           "latency_by_size")},
            "full_stream": {"solves": count * (full_steps + 1), "wall_s": full_s,
                            "solves_per_s": count * (full_steps + 1) / full_s},
            "cost_model": {"requests_measured": len(meas), "measure_s": t_meas,
                           "loo_rel_err_median": float(np.median(loo)),
                           "loo_rel_err_max": float(np.max(loo))},
        }
    ratio = lambda a, b: a / b if b else None  # noqa: E731
    same, fast = plain["plain_same_config"], plain["plain_fast_equal_error"]
    work_small = sum(r.n for r in base if r.n < 100_000) / total_n
    return {
        "workload": f"{count} requests ({total_n:,} particles), Poisson {rate:.0f}/s, N "
                    f"log-uniform in [1e3, 2e6], half Plummer half uniform cubes, {steps} KDK "
                    "steps each (dt 1e-3, eps 0.01), refit every step, rebuild every 10, HBM "
                    f"budget {hbm_budget / 1e9:.0f} GB",
        "server_config": {"form": "fp32", "theta": theta, "criterion": criterion,
                          "multipole": multipole, "leaf_size": leaf,
                          "scheduling": "shortest remaining work first",
                          "solve_budget_particles": solve_budget},
        "server_stream_window": st,
        "server_full_stream": full_server,
        "full_stream_steps": full_steps,
        **plain,
        "solves_per_s_ratio_full_stream_vs_same_config": ratio(
            full_server["solves_per_s"], same["full_stream"]["solves_per_s"]),
        "solves_per_s_ratio_full_stream_vs_fast": ratio(
            full_server["solves_per_s"], fast["full_stream"]["solves_per_s"]),
        "solves_in_window_ratio_vs_same_config": ratio(st["solves"],
                                                       same["stream_window"]["solves"]),
        "solves_in_window_ratio_vs_fast": ratio(st["solves"], fast["stream_window"]["solves"]),
        "work_share_of_systems_below_1e5": work_small,
        "median_err_vs_fp64_direct": {
            "server_and_plain_same_config": float(np.median(e_srv)),
            f"plain_fast_theta_{fast_theta}": float(np.median(e_fast)),
            "plain_fast_theta_0.5": float(np.median(e_fast05)),
            "requests_n": [r.n for r in pick]},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("report", choices=["precision", "batched", "served", "scaling", "build"])
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--sizes", default="1e5,1e6,4e6,16e6,64e6")
    ap.add_argument("--count", type=int, default=24)
    ap.add_argument("--nsys", type=int, default=2048)
    ap.add_argument("--n", type=int, default=None,
                    help="particles (precision: 4,000,000; build: 1,000,000)")
    ap.add_argument("--sample", type=int, default=8192)
    ap.add_argument("--criterion", default=None)
    ap.add_argument("--multipole", default=None)
    ap.add_argument("--theta", type=float, default=None)
    ap.add_argument("--thetas", default="0.3,0.5,0.7")
    ap.add_argument("--plain-theta-equal", type=float, default=None)
    args = ap.parse_args()
    if args.report == "precision":
        precision_report(args.n or 4_000_000, args.sample, criterion=args.criterion or "bh",
                         multipole=args.multipole or "mono",
                         thetas=tuple(float(x) for x in args.thetas.split(",")))
    elif args.report == "batched":
        batched_report(args.nsys, criterion=args.criterion or "bh",
                       multipole=args.multipole or "mono",
                       theta=args.theta if args.theta is not None else 0.5)
    elif args.report == "build":
        build_report(args.n or 1_000_000, args.reps)
    elif args.report == "scaling":
        scaling_report(tuple(int(float(x)) for x in args.sizes.split(",")))
    elif args.report == "served":
        served_report(args.count, criterion=args.criterion or "bh_offset",
                      multipole=args.multipole or "quad",
                      theta=args.theta if args.theta is not None else 0.7,
                      plain_theta_equal_error=args.plain_theta_equal)


if __name__ == "__main__":
    main()
