"""Benchmark: Barnes-Hut self accelerations of a 1,000,000-particle Plummer
sphere (theta=0.5, softening=0.01, G=1, leaf_size=32) on one GB300.

One step = one full solve through a persistent tree handle: bounding box,
Morton keys, radix sort, gather, bottom-up node moments, and the traversal
over all N targets (what bhut.Tree.rebuild + Tree.accelerations do), with
inputs already resident in HBM.  ``e2e`` repeats the metric through the
public API (``bhut_gb300.accelerations``) with host NumPy buffers, so the
host<->device copies are inside its timed region.

The same line carries bounded sub-records of the other named workloads:
``c1`` (10,000 Gaussian particles, the reference's CPU-runnable case),
``exact`` (the IEEE-FP64 form at the headline workload), ``batched`` (2,048
Plummer systems in one graph solve), ``precision`` (4M galaxy, FP32 form,
three thetas) and ``served`` (200-request Poisson stream against the plain
per-request path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form exact|fast|fp32]
    python bench.py --impl reference ...   # the reference's algorithm on the host cores

Under torchrun (N > 1) every rank solves its own system (replicas; the
path has no exchange step), times are maxed over ranks and rank 0 prints
one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "accels/s N=1M θ=0.5; served solves/s & p99 vs plain GPU at equal FP64 err"
N_DEFAULT = 1_000_000
THETA, EPS, G, LEAF = 0.5, 0.01, 1.0, 32
FLOPS_PER_INTERACTION = 20  # conventional N-body count per pair/monopole evaluation


def _workload_desc(n, form):
    return {
        "workload": f"Plummer sphere N={n:,} (a=1, radii truncated at 20a, equal masses 1/N, "
                    f"seed 1+rank), self accelerations: tree build + Barnes-Hut traversal",
        "n": n, "theta": THETA, "softening": EPS, "G": G, "leaf_size": LEAF, "form": form,
        "l2": "512 MiB buffer written between timed steps (L2 flush)",
    }


# ---------------------------------------------------------------------------
# process group (replicas only: barrier + max of times, no data-path traffic)
# ---------------------------------------------------------------------------
def _dist(gpu: bool = True):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            # NCCL with one GPU per rank; gloo for CPU-only runs (the
            # reference arm) or when ranks share a GPU
            import torch
            nccl = gpu and torch.cuda.is_available() and torch.cuda.device_count() >= ws
            if nccl:
                torch.cuda.set_device(local)
            dist.init_process_group("nccl" if nccl else "gloo")
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU side: the oracle (scalar FP64 restatement of the reference's path)
# ---------------------------------------------------------------------------
def host_threads() -> int:
    """Every host core this process may run on (torchrun sets
    OMP_NUM_THREADS=1, which must not shrink the CPU baseline)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_solve_sample(pos, m, sample_targets: int, seed: int = 0) -> dict:
    """Times the oracle on the host: full tree build (serial, as the
    reference's build) plus the traversal of a bounded random sample of
    targets on all host threads; returns the extrapolated whole-job rate."""
    from oracle import oracle
    n = len(pos)
    t0 = time.perf_counter()
    tree = oracle.build_tree(pos, m, LEAF)
    t_build = time.perf_counter() - t0
    idx = np.random.default_rng(seed).choice(n, min(sample_targets, n), replace=False)
    t0 = time.perf_counter()
    threads = host_threads()
    oracle.accelerations(tree, pos, m, theta=THETA, softening=EPS, G=G, self_index=idx,
                         nthreads=threads)
    t_trav = time.perf_counter() - t0
    per_target = t_trav / len(idx)
    total = t_build + per_target * n
    return {"value": n / total, "t_build_s": t_build, "t_sample_s": t_trav,
            "sample_targets": len(idx), "cores": threads}


def cpu_solve_all(pos, m, acc_gpu) -> dict:
    """The oracle's full solve (serial build, traversal of every target on
    all host threads) of a small workload, timed; with the relative L2
    difference of the GPU result from it."""
    from oracle import oracle
    threads = host_threads()
    t0 = time.perf_counter()
    tree = oracle.build_tree(pos, m, LEAF)
    ref = oracle.accelerations(tree, pos, m, theta=THETA, softening=EPS, G=G, nthreads=threads)
    t = time.perf_counter() - t0
    rel = float(np.linalg.norm(acc_gpu - ref) / np.linalg.norm(ref))
    return {"value": len(pos) / t, "unit": "accels/s", "cores": threads, "kind": "port",
            "sample": f"oracle (C restatement of the reference's path): full solve of all "
                      f"{len(pos):,} targets, {t:.3f} s",
            "gpu_rel_l2_vs_oracle": rel}


def run_reference(args, ws, rank):
    """--impl reference: the reference's algorithm (oracle port, C, OpenMP on
    every host core) on the same workload; rank 0 only."""
    if rank != 0:
        return
    from bhut_gb300 import workloads
    from oracle import oracle
    oracle.build()
    pos, m = workloads.plummer(args.n, seed=1)
    sample = args.ref_sample
    # calibrate the sample so that one step stays near 2 s of traversal
    probe = cpu_solve_sample(pos, m, 512, seed=99)
    rate = probe["sample_targets"] / max(probe["t_sample_s"], 1e-9)
    if sample <= 0:
        sample = int(min(args.n, max(1024, rate * 2.0)))
    for w in range(args.warmup):
        cpu_solve_sample(pos, m, sample, seed=w)
    vals, build_s = [], []
    t0 = time.perf_counter()
    for k in range(args.steps):
        r = cpu_solve_sample(pos, m, sample, seed=100 + k)
        vals.append(r["value"])
        build_s.append(r["t_build_s"])
    wall = time.perf_counter() - t0
    value = float(statistics.mean(vals))
    cores = host_threads()
    desc = (f"per step: full serial tree build of N={args.n:,} plus the traversal of {sample} "
            f"random targets on {cores} threads; accels/s = N / (build time + N x per-target "
            f"traversal time)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "accels/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": _workload_desc(args.n, "oracle-port"),
        "cpu_baseline": {"value": value, "unit": "accels/s", "cores": cores, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": "accels/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "build_s_mean": float(statistics.mean(build_s)),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def measure_gemm_peak(torch, dtype) -> float:
    """Measured dense throughput of this GPU for one precision: cuBLAS GEMM
    (torch.matmul, TF32 disabled for float32), 4096^3, best of 5, TFLOP/s."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 4096
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


# Instructions of one float-float pair (or monopole) term of the fast form,
# counted from bhut_gb300/csrc/fast.cuh (pair_ff_soft, 3-D, target inside
# the box, softening bounding R from below as in this workload): exact
# displacement and squares 21, cross term and r^2 low part 4, three
# non-negative FastTwoSums into r^2 21 (6 of them min/max on the ALU pipe),
# MUFU rsqrt 1, refinement and cube 10, three float-float products and
# magnitude-ordered two-sum accumulations 36 (9 compare/select on the ALU
# pipe) -> 93 for a leaf pair in the unit-mass frame (every particle the same
# mass), 97 with the mass product (monopoles, or unequal masses).  Of these,
# 77 / 81 run on the FP32 (FMA) pipe.  The fp32 form's counts live in
# bhut_gb300.reports.
FF_INSTR_UNIT_PAIR, FF_INSTR_MASS_PAIR = 93, 97
FF_FMA_UNIT_PAIR, FF_FMA_MASS_PAIR = 77, 81
ARITH = {"exact": "IEEE FP64",
         "fast": "float-float on the FP32 pipe (about 48-bit significand); FP64 bounding box, "
                 "keys, centres of mass and rare fallbacks",
         "fp32": "FP32 + Kahan; FP64 bounding box, keys and centres of mass"}
DTYPE = {"exact": "f64", "fast": "f64-ff", "fp32": "f32"}
# Algorithmic bytes of one rebuild (the build kernels' compulsory reads and
# writes): per particle staging copy + box 64, Morton keys 36, digit
# histograms 8, eight sort passes 8 x 24, Morton-ordered gather 68, leaf
# moments 32; per node about 200 (moments, boxes, links of both children
# read, its own written).
BUILD_BYTES_PER_PARTICLE = 64 + 36 + 8 + 8 * 24 + 68 + 32
BUILD_BYTES_PER_NODE = 200


def run_ours(args, ws, rank, local):
    import torch
    import bhut_gb300 as bh
    from bhut_gb300 import _lib, workloads
    from bhut_gb300.api import _Handle

    # one GPU per local rank; on a node with fewer GPUs than ranks the ranks
    # share them (replicas never wait on one another)
    local = local % max(torch.cuda.device_count(), 1)
    torch.cuda.set_device(local)
    L = _lib.load()
    n = args.n
    pos, m = workloads.plummer(n, seed=1 + rank)
    pos_d = torch.from_numpy(pos).cuda()
    m_d = torch.from_numpy(m).cuda()
    out_d = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    h = _Handle(3, LEAF, stream=stream.cuda_stream)
    h.set_form(args.form)

    def step():
        h.rebuild(pos_d, m_d)
        ev_mid = torch.cuda.Event(enable_timing=True)
        ev_mid.record(stream)
        h.accel_self(THETA, EPS, G, out_d)
        return ev_mid

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        step()
    torch.cuda.synchronize()
    p2p, m2p, visits = h.stats()
    fb_dec, fb_pairs = h.fallbacks()

    clocks = ClockSampler(local)
    _barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = L.bhut_launch_count()
    total_ms, trav_ms = 0.0, 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mid = step()
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        trav_ms += mid.elapsed_time(e1)
    torch.cuda.synchronize()
    launches = L.bhut_launch_count() - launches0
    clk = clocks.stop()
    _barrier(ws)
    t_max = _max_over_ranks(total_ms / 1e3, ws)
    value = ws * n * args.steps / t_max

    # end to end through the public API with host buffers (one untimed call,
    # then e2e_steps timed calls)
    e2e_steps = max(1, args.e2e_steps)
    bh.accelerations(pos, m, theta=THETA, softening=EPS, G=G, leaf_size=LEAF, form=args.form)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        acc = bh.accelerations(pos, m, theta=THETA, softening=EPS, G=G, leaf_size=LEAF,
                               form=args.form)
    torch.cuda.synchronize()
    t_e2e = _max_over_ranks(time.perf_counter() - t0, ws)
    e2e_value = ws * n * e2e_steps / t_e2e
    assert np.all(np.isfinite(acc))

    if rank != 0:
        h.close()
        return
    hbm_peak = _measured_hbm_gbs()
    peak64 = measure_gemm_peak(torch, torch.float64)
    peak32 = measure_gemm_peak(torch, torch.float32)
    ffma = ctypes.c_double(0.0)
    _lib.check(L.bhut_measure_fp32_peak(ctypes.byref(ffma)))
    ffma_tflops = ffma.value
    trav_s = trav_ms / 1e3 / args.steps
    inter = p2p + m2p
    flops = FLOPS_PER_INTERACTION * inter
    achieved64 = flops / trav_s / 1e12
    traffic = _traffic_from_profile(args)
    if args.form == "exact":
        roofline = {
            "bound": "fp64", "kernel": "k_traverse_exact", "achieved": achieved64,
            "peak": peak64, "unit": "TFLOP/s", "frac": achieved64 / peak64, "traffic": traffic,
            "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (MEASURED_PEAKS.json has "
                           "no FP64 figure)",
            "work_per_launch": flops,
            "work_rule": f"{FLOPS_PER_INTERACTION} flop x (pair + monopole evaluations counted "
                         "by the kernel)"}
    else:
        if args.form == "fast":
            unit = bool(m[0] > 0 and np.all(m == m[0]))
            ipair = FF_INSTR_UNIT_PAIR if unit else FF_INSTR_MASS_PAIR
            fpair = FF_FMA_UNIT_PAIR if unit else FF_FMA_MASS_PAIR
            ops = ipair * p2p + FF_INSTR_MASS_PAIR * m2p
            fma_ops = fpair * p2p + FF_FMA_MASS_PAIR * m2p
            rule = (f"{ipair} pair-term instructions per leaf pair{' (unit-mass frame)' if unit else ''}"
                    f", {FF_INSTR_MASS_PAIR} per monopole (FP32 + ALU + MUFU; one warp "
                    "instruction per clock per SM sub-partition is both the issue limit and "
                    "the FFMA rate below)")
        else:
            from bhut_gb300 import reports
            ops = reports.fp32_ops(p2p, m2p, "mono")
            rule = (f"{reports.F32_OPS_PER_PAIR} FP32 ops per pair term (unit-mass frame), "
                    f"{reports.F32_OPS_PER_MONOPOLE} per Kahan-added monopole")
        achieved32 = ops / trav_s / 1e12
        # FP32 pipe lane-instructions per second (one FMA = 2 flop): the FMA
        # chains of bhut_measure_fp32_peak, and cuBLAS SGEMM for comparison
        fma_rate = ffma_tflops / 2.0
        sgemm_rate = peak32 / 2.0
        roofline = {
            "bound": "fp32",
            "kernel": "k_traverse_fast" if args.form == "fast" else "k_traverse_fp32",
            "achieved": achieved32,
            "peak": fma_rate,
            "unit": "T instr/s" if args.form == "fast" else "T FP32-pipe ops/s",
            "frac": achieved32 / fma_rate,
            "traffic": traffic,
            "peak_source": "independent FP32 FMA chains on every SM, measured in this run "
                           "(bhut_measure_fp32_peak); MEASURED_PEAKS.json has no FP32 figure",
            "peak_sgemm": sgemm_rate, "frac_vs_sgemm": achieved32 / sgemm_rate,
            "peak_sgemm_source": "cuBLAS SGEMM 4096^3 (TF32 off) measured in this run, / 2",
            "work_per_launch": ops,
            "work_rule": f"{rule} x evaluations counted by the kernel",
            **({"fp32_pipe_frac": fma_ops / trav_s / 1e12 / fma_rate,
                "fp32_pipe_rule": f"{fpair} FP32-pipe ops per leaf pair, {FF_FMA_MASS_PAIR} per "
                                  "monopole, against the same FFMA rate"}
               if args.form == "fast" else {}),
            "fp64_equivalent": {"achieved": achieved64, "peak": peak64, "unit": "TFLOP/s",
                                "frac": achieved64 / peak64,
                                "rule": f"{FLOPS_PER_INTERACTION} flop per interaction vs "
                                        "measured DGEMM"}}
    build_s = (total_ms - trav_ms) / args.steps / 1e3
    m_nodes = h.info()[1]
    build_bytes = BUILD_BYTES_PER_PARTICLE * n + BUILD_BYTES_PER_NODE * m_nodes
    line = {
        "metric": METRIC, "value": value, "unit": "accels/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE[args.form], "arith": ARITH[args.form],
        "data": "synthetic", "config": _workload_desc(n, args.form),
        "e2e": {"value": e2e_value, "unit": "accels/s",
                "h2d_bytes_per_step": int(pos.nbytes + m.nbytes),
                "d2h_bytes_per_step": int(n * 3 * 8), "api": "bhut_gb300.accelerations",
                "timed_calls": e2e_steps, "untimed_calls_before": 1},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "traversal_ms": trav_s * 1e3,
        "build_ms": build_s * 1e3,
        "roofline_build": {"bound": "hbm", "achieved": build_bytes / build_s / 1e9,
                           "peak": hbm_peak, "unit": "GB/s",
                           "frac": build_bytes / build_s / 1e9 / hbm_peak,
                           "bytes_per_rebuild": int(build_bytes),
                           "bytes_rule": f"{BUILD_BYTES_PER_PARTICLE} B per particle + "
                                         f"{BUILD_BYTES_PER_NODE} B per node (compulsory "
                                         "reads and writes of the build kernels)",
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)",
                           "note": "build_ms is the device time from the start of the "
                                   "rebuild call to the start of the traversal, host "
                                   "round trips (input check, error word) included"},
        "interactions_per_solve": {"p2p": p2p, "m2p": m2p, "node_visits": visits,
                                   "fp64_fallback_decisions": fb_dec, "fp64_pairs": fb_pairs},
        "clocks": clk,
    }
    c1 = None
    if ws == 1 and not args.quick:
        from bhut_gb300 import reports
        fma_rate = ffma_tflops / 2.0
        if not args.no_c1:
            c1 = reports.c1_record(fma_rate=fma_rate)
            line["c1"] = c1[0]
        if not args.no_c2_sequence:
            line["c2_sequence"] = reports.c2_sequence_record(pos_d, m_d, theta=THETA, eps=EPS,
                                                             G=G, leaf=LEAF)
        if not args.no_exact:
            line["exact"] = reports.exact_record(pos_d, m_d, theta=THETA, eps=EPS, G=G,
                                                 leaf=LEAF, fp64_peak=peak64)
        if not args.no_batched:
            line["batched"] = reports.batched_record(fma_rate=fma_rate)
        if not args.no_precision:
            line["precision"] = reports.precision_record(fma_rate=fma_rate)
        if not args.no_served:
            line["served"] = reports.served_record(
                count=args.served_count, server_seconds=args.served_seconds)
    if not args.no_cpu_baseline:
        cb = cpu_solve_sample(pos, m, args.cpu_sample)
        line["cpu_baseline"] = {
            "value": cb["value"], "unit": "accels/s", "cores": cb["cores"], "kind": "port",
            "sample": f"oracle (C restatement of the reference's path): full serial build of "
                      f"N={n:,} ({cb['t_build_s']:.2f} s) + traversal of "
                      f"{cb['sample_targets']} random targets ({cb['t_sample_s']:.2f} s, "
                      f"{cb['cores']} threads), extrapolated to N targets"}
        if c1 is not None:
            line["c1"]["cpu_baseline"] = cpu_solve_all(*c1[2], c1[1])
    h.close()
    print(json.dumps(line), flush=True)


def _measured_hbm_gbs() -> float:
    """HBM copy bandwidth measured on this machine (MEASURED_PEAKS.json), else
    the stated fallback."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def _traffic_from_profile(args):
    """DRAM bytes per traversal launch from the committed ncu summary, if any."""
    path = os.path.join(HERE, "profiles", f"traversal_{args.form}_dram.json")
    try:
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_launch_scaled")
    except (OSError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["exact", "fast", "fp32"], default=None)
    ap.add_argument("--n", "--particles", dest="n", type=int, default=N_DEFAULT,
                    help="particles (--particles under torchrun, whose parser takes --n)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-sample", type=int, default=16384)
    ap.add_argument("--ref-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="headline only: no exact, batched, precision or served sub-record")
    ap.add_argument("--no-exact", action="store_true")
    ap.add_argument("--no-c2-sequence", action="store_true",
                    help="skip the external-target / refit / rebuild record of the 1M workload")
    ap.add_argument("--no-c1", action="store_true",
                    help="skip the 10,000-particle Gaussian sub-record")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-served", action="store_true",
                    help="skip the served-stream comparison (about two minutes)")
    ap.add_argument("--served-count", type=int, default=200)
    ap.add_argument("--served-seconds", type=float, default=45.0,
                    help="window of the open-loop stream comparison")
    args = ap.parse_args()
    if args.form is None:
        from bhut_gb300.api import DEFAULT_FORM
        args.form = DEFAULT_FORM
    ws, rank, local = _dist(gpu=args.impl != "reference")
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
