"""Served form: continuous batching of N-body systems with device-resident state.

A request is one N-body system (positions, velocities, masses) to advance by
``steps`` kick-drift-kick leapfrog steps.  The server keeps every admitted
system's state in HBM and advances all of them together, one batched solve
per tick:

* admission: a queued request is admitted at a tick boundary once it has
  arrived and its device footprint (``bytes_per_particle``: the buffers
  counted, plus a measured allocator margin) fits the HBM budget (and the
  optional cap on resident particles); a request that does not fit even on an
  empty server is rejected;
* each tick: first half-kick and drift (``bhut_leapfrog``), one batched
  solve (``bhut_batch_*``), second half-kick, for the systems that run this
  tick.  With a per-solve particle budget (``solve_budget``) the running
  systems are chosen shortest remaining work first (particles x remaining
  steps), greedily up to the budget (at least one system), so small
  requests do not wait for the largest resident system at every step;
  the others keep their state in HBM and wait.  The choice is revisited at
  every admission and retirement.  Without a budget every resident system
  steps every tick;
* each system refits its tree on its own schedule -- its Morton order is kept
  (``bhut_batch_keep_order``) and node boxes and moments are recomputed --
  and rebuilds it every ``rebuild_every`` of its own steps, or earlier when a
  particle leaves 1.1x the root box of its last rebuild (the reference's
  refit-vs-rebuild test, ``bhut_batch_outside``).  Nothing a system
  computes depends on which other systems share the batch, so a request's
  trajectory is the same alone and in any mix (bit for bit);
* a finished request leaves at the next tick boundary and frees its slot; so
  does a cancelled one (``Server.cancel``) and one past its deadline
  (``Request.deadline`` seconds after arrival), queued or resident, without
  changing any other request's trajectory;
* latency = completion time - arrival time (queueing included), over the
  requests that finished;
* ``snapshot``/``restore`` copy the queued and resident requests' state
  (positions, velocities, accelerations, Morton order, step counts) to host
  memory and back; a restored server continues every trajectory bit for bit.

``plain_path`` runs the same stream the simple way for comparison: one
request at a time, one ``Tree`` per request (form ``fast``), ``refit`` every
step and ``rebuild`` every ``rebuild_every`` steps.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib, api, workloads
from .batch import BatchedSolver

# Device bytes per resident particle, counted from the buffers:
#  request state: x, v, a (3 x 24), m (8), last Morton order (4), and the same
#    again while the packed arrays are rebuilt after an admission/retirement;
#  batch: positions and masses copies (32), keys, second keys (16), perm and
#    system ids (8), sorted SoA (32), float-float copies (32), sort scratch
#    (12), kept-order and tick permutations (12);
#  nodes: about 2 N / leaf_size of 268 B (centre of mass and mass 32, size,
#    half, centre, AABB scratch 88, topology links 20, float-float copies and
#    header 56, quadrupoles and their float copies 72).
STATE_BYTES = 2 * (3 * 24 + 8 + 4)
BATCH_BYTES = 32 + 16 + 8 + 32 + 32 + 12 + 12
NODE_BYTES = 268
# allocator granularity, buffers kept at their largest layout and the copies
# made while repacking, on top of the buffer count: measured 1.16x at a steady
# 3.1M resident particles and 1.87x over a 100-request stream with admissions
# and retirements every few ticks (device memory above the server's start,
# leaf 16)
FOOTPRINT_MARGIN = 2.0


def bytes_per_particle(leaf_size: int) -> float:
    return FOOTPRINT_MARGIN * (STATE_BYTES + BATCH_BYTES + 2.0 * NODE_BYTES / leaf_size)


def admits(resident: int, n_active: int, n: int, *, leaf_size: int, hbm_budget: float,
           max_active: int | None = None) -> bool:
    """Admission rule: a request of ``n`` particles joins ``n_active``
    resident systems holding ``resident`` particles when the estimated device
    footprint of all of them fits ``hbm_budget`` bytes and, with a cap, the
    resident particle count stays within ``max_active`` (a request alone on
    an empty server is always admitted past the cap, never past the budget)."""
    if max_active is not None and n_active and resident + n > max_active:
        return False
    return (resident + n) * bytes_per_particle(leaf_size) <= hbm_budget


def retire_reason(steps_done: int, steps: int, waited: float, deadline: float | None,
                  cancelled: bool) -> str | None:
    """Why a request leaves at this tick boundary, if it does: "cancelled",
    "done" (all its steps taken), "timed_out" (``waited`` seconds since its
    arrival exceed its ``deadline``), else None."""
    if cancelled:
        return "cancelled"
    if steps_done >= steps:
        return "done"
    if deadline is not None and waited > deadline:
        return "timed_out"
    return None


def remaining_work(n: int, steps: int, steps_done: int, primed: bool) -> int:
    """Particle-solves a request still needs: one per remaining step, plus
    the initial force evaluation if it has not run yet."""
    return n * (max(steps - steps_done, 0) + (0 if primed else 1))


def choose_running(work: list[tuple[int, int, int]], budget: int | None) -> list[int]:
    """Which resident systems step in the next solve.  ``work`` holds
    (remaining work, particles, request id) per resident system; returns
    positions in ``work``.  Without a budget: all of them.  With one:
    shortest remaining work first (ties by request id), each system taken
    while the running particle total stays within ``budget``; the first is
    always taken, so a system larger than the budget still runs."""
    if budget is None:
        return list(range(len(work)))
    order = sorted(range(len(work)), key=lambda k: (work[k][0], work[k][2]))
    chosen, total = [], 0
    for k in order:
        n = work[k][1]
        if chosen and total + n > budget:
            continue
        chosen.append(k)
        total += n
    return sorted(chosen)


def size_class(n: int) -> str:
    """Latency report classes by particle count."""
    return "n<1e4" if n < 10_000 else ("1e4<=n<1e5" if n < 100_000 else "n>=1e5")


def latency_summary(items: list[tuple[int, float]]) -> dict:
    """p50/p99 latency overall and per size class from (particles,
    latency) of finished requests."""
    def stats(lat):
        a = np.asarray(lat, dtype=float)
        return {"count": int(a.size),
                "p50_s": float(np.percentile(a, 50)) if a.size else None,
                "p99_s": float(np.percentile(a, 99)) if a.size else None}
    out = {"all": stats([t for _, t in items])}
    for cls in ("n<1e4", "1e4<=n<1e5", "n>=1e5"):
        out[cls] = stats([t for n, t in items if size_class(n) == cls])
    return out


def keeps_order(primed: bool, has_order: bool, steps_done: int, rebuild_every: int) -> bool:
    """Refit (keep the last Morton order) unless this system's rebuild is
    due: its first solve, and every ``rebuild_every`` of its own steps
    (bhut's Tree.refit / Tree.rebuild schedule of the served workload)."""
    return primed and has_order and steps_done % rebuild_every != 0


@dataclass
class Request:
    rid: int
    arrival: float
    positions: np.ndarray
    velocities: np.ndarray
    masses: np.ndarray
    steps: int = 100
    kind: str = ""
    deadline: float | None = None   # seconds after arrival; None: no deadline
    # runtime state
    status: str = ""                # "done", "cancelled", "timed_out" or "rejected" once it left
    steps_done: int = 0
    solves: int = 0
    primed: bool = False
    admitted_at: float | None = None
    done_at: float | None = None
    order: object = None          # local Morton order of the last solve (device int32)
    root: object = None           # root centre and half-size at the last rebuild
    forced_rebuilds: int = 0      # rebuilds forced by particles leaving the root box
    forced_seen: int = 0          # of those, already counted from the solver's counter
    slot: tuple = field(default=(0, 0))
    acc: object = None

    @property
    def n(self) -> int:
        return len(self.masses)

    @property
    def latency(self) -> float | None:
        return None if self.done_at is None else self.done_at - self.arrival


def request_stream(count: int, *, rate: float = 200.0, nmin: int = 1000, nmax: int = 2_000_000,
                   steps: int = 100, seed: int = 0, vel_sigma: float = 0.1) -> list[Request]:
    """Poisson arrivals (mean ``rate`` per second); N log-uniform in
    [nmin, nmax]; half Plummer spheres (a = 1), half uniform cubes of side 2;
    equal masses 1/N; velocities N(0, vel_sigma^2) per component."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        sd = int(rng.integers(0, 2**31 - 1))
        if rng.random() < 0.5:
            pos, m = workloads.plummer(n, seed=sd)
            kind = "plummer"
        else:
            pos, m = workloads.uniform_cube(n, seed=sd, side=2.0)
            kind = "cube"
        vel = np.random.default_rng(sd + 1).normal(0.0, vel_sigma, (n, 3))
        out.append(Request(i, float(t[i]), pos, vel, m, steps=steps, kind=kind))
    return out


def _leapfrog(L, pos, vel, acc, n, kick, drift, stream):
    _lib.check(L.bhut_leapfrog(pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), int(n), 3,
                               float(kick), float(drift), stream))


class Server:
    """Continuous-batching server; see the module docstring."""

    def __init__(self, *, theta: float = 0.5, softening: float = 0.01, G: float = 1.0,
                 dt: float = 1e-3, rebuild_every: int = 10, form: str = "fp32",
                 criterion: str = "bh_offset", leaf_size: int = 16, targets_per_warp: int = 32,
                 hbm_budget: float = 150e9, max_active_particles: int | None = None,
                 multipole: str = "quad", solve_budget: int | None = None):
        import torch
        self.torch = torch
        self.theta, self.eps, self.G, self.dt = theta, softening, G, dt
        self.rebuild_every = rebuild_every
        self.leaf_size = leaf_size
        self.hbm_budget = hbm_budget
        self.max_active = max_active_particles
        self.solve_budget = solve_budget
        self.running: list[Request] = []   # the resident systems that step each tick
        self.L = _lib.load()
        self.stream = torch.cuda.current_stream().cuda_stream
        self.solver = BatchedSolver(dim=3, leaf_size=leaf_size, form=form, criterion=criterion,
                                    targets_per_warp=targets_per_warp, use_graph=False,
                                    stream=self.stream, multipole=multipole)
        # the refit-vs-rebuild test runs inside each solve (no host round trip)
        _lib.check(self.L.bhut_batch_set_refit_rule(self.solver.h, 1))
        self.packed: list[Request] = []    # systems of the solver's current layout, in order
        self._roots_dirty = False
        self.active: list[Request] = []
        self.finished: list[Request] = []
        self.ticks = 0
        self._solve_events = []
        self._cancel: set[int] = set()
        self.queue: list[Request] = []
        self.mem_peak = 0
        # device memory in use before any request state (the reported peak
        # is measured against it)
        torch.cuda.synchronize()
        free, total = torch.cuda.mem_get_info()
        self.mem_base = total - free
        self.solves = 0
        self.accels = 0
        self.peak_bytes = 0.0

    # -- device state ------------------------------------------------------
    def cancel(self, rid: int) -> None:
        """Cancels request ``rid`` (queued or resident) at the next tick
        boundary."""
        self._cancel.add(rid)

    def _fits(self, r: Request) -> bool:
        return admits(sum(a.n for a in self.active), len(self.active), r.n,
                      leaf_size=self.leaf_size, hbm_budget=self.hbm_budget,
                      max_active=self.max_active)

    def _sync_roots(self) -> None:
        """Copies the solver's per-system root boxes and forced-rebuild counts
        of the current layout back into the requests (one host round trip)."""
        if not self.packed or self._roots_dirty:
            return
        ns = len(self.packed)
        roots = np.zeros((ns, 4))
        forced = np.zeros(ns, dtype=np.int32)
        _lib.check(self.L.bhut_batch_roots(self.solver.h, roots.ctypes.data))
        _lib.check(self.L.bhut_batch_forced(self.solver.h, forced.ctypes.data))
        for k, r in enumerate(self.packed):
            if r.primed:
                r.root = roots[k].copy()
            r.forced_rebuilds += int(forced[k]) - r.forced_seen
            r.forced_seen = int(forced[k])

    def _pack(self):
        """Chooses the running systems and concatenates their state into one
        set of device arrays (after an admission or a retirement).  Resident
        systems that do not run keep a private copy of their state."""
        torch = self.torch
        self._sync_roots()
        dev = "cuda"
        work = [(remaining_work(r.n, r.steps, r.steps_done, r.primed), r.n, r.rid)
                for r in self.active]
        self.running = [self.active[k] for k in choose_running(work, self.solve_budget)]
        running = set(id(r) for r in self.running)
        packed = set(id(r) for r in self.packed)
        for r in self.active:
            if id(r) not in running and id(r) in packed:   # leaves the packed arrays
                r.positions, r.velocities = r.positions.clone(), r.velocities.clone()
                r.acc, r.masses = r.acc.clone(), r.masses.clone()
                if r.order is not None:
                    r.order = r.order.clone()
        parts_x, parts_v, parts_a, parts_m = [], [], [], []
        for r in self.running:
            parts_x.append(r.positions)
            parts_v.append(r.velocities)
            parts_a.append(r.acc)
            parts_m.append(r.masses)
        self.x = torch.cat(parts_x).contiguous()
        self.v = torch.cat(parts_v).contiguous()
        self.a = torch.cat(parts_a).contiguous()
        self.m = torch.cat(parts_m).contiguous()
        sizes = [r.n for r in self.running]
        self.off = np.zeros(len(sizes) + 1, dtype=np.int64)
        self.off[1:] = np.cumsum(sizes)
        for k, r in enumerate(self.running):         # views into the packed arrays
            s, e = int(self.off[k]), int(self.off[k + 1])
            r.positions, r.velocities, r.acc, r.masses = self.x[s:e], self.v[s:e], self.a[s:e], \
                self.m[s:e]
            r.slot = (s, e)
        self.perm = torch.empty(int(self.off[-1]), dtype=torch.int32, device=dev)
        self.packed = list(self.running)
        self._roots_dirty = True
        self.peak_bytes = max(self.peak_bytes, float(sum(r.n for r in self.active)) *
                              bytes_per_particle(self.leaf_size))

    # -- one tick ------------------------------------------------------------
    def tick(self) -> None:
        torch = self.torch
        dt = self.dt
        for r in self.running:                       # first half-kick + drift
            if r.primed:
                _leapfrog(self.L, r.positions, r.velocities, r.acc, r.n, 0.5 * dt, dt,
                          self.stream)
        keep = np.zeros(len(self.running), dtype=np.uint8)
        perm_in = None
        for k, r in enumerate(self.running):         # refit unless a rebuild is due
            if keeps_order(r.primed, r.order is not None, r.steps_done, self.rebuild_every):
                keep[k] = 1
        self.solver.load(self.x, self.m, self.off)
        if self._roots_dirty:
            # a new layout: its systems' root boxes (those never rebuilt are
            # not kept anyway), forced-rebuild counters from zero.  Inside the
            # solve a kept system that has a particle beyond 1.1x its root box
            # is rebuilt (should_refit_vs_rebuild, bhut/tree/refit.py:236-249).
            roots = np.zeros((len(self.running), 4))
            for k, r in enumerate(self.running):
                if r.root is not None:
                    roots[k] = r.root
                r.forced_seen = 0
            _lib.check(self.L.bhut_batch_set_roots(self.solver.h, roots.ctypes.data))
            self._roots_dirty = False
        if keep.any():
            perm_in = torch.cat([
                (r.order + int(self.off[k])) if r.order is not None
                else torch.zeros(r.n, dtype=torch.int32, device="cuda")
                for k, r in enumerate(self.running)])
            _lib.check(self.L.bhut_batch_keep_order(self.solver.h, keep.ctypes.data,
                                                    perm_in.data_ptr()))
        else:
            _lib.check(self.L.bhut_batch_keep_order(self.solver.h, None, None))
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        self.solver.solve(theta=self.theta, softening=self.eps, G=self.G, out=self.a)
        ev1.record()
        self._solve_events.append((ev0, ev1))
        _lib.check(self.L.bhut_batch_order(self.solver.h, self.perm.data_ptr()))
        for k, r in enumerate(self.running):
            s, e = r.slot
            r.order = self.perm[s:e] - s
            if r.primed:                            # second half-kick
                _leapfrog(self.L, r.positions, r.velocities, r.acc, r.n, 0.5 * dt, 0.0,
                          self.stream)
                r.steps_done += 1
            else:
                r.primed = True                     # a(0): the initial force evaluation
            r.solves += 1
        self.solves += len(self.running)
        self.accels += int(self.off[-1])
        self.ticks += 1

    # -- the loop ----------------------------------------------------------
    def _leave(self, r: Request, reason: str, t: float) -> None:
        r.status = reason
        r.done_at = t
        self.finished.append(r)
        if r.primed or r.admitted_at is not None:
            # the response goes to host memory and frees its device slot
            r.final_positions = r.positions.to("cpu")
            r.final_velocities = r.velocities.to("cpu")

    def run(self, requests: list[Request] = (), *, realtime: bool = True,
            max_seconds: float | None = None, max_ticks: int | None = None,
            t0: float = 0.0) -> dict:
        """Serves ``requests`` (plus any restored queue) until all have left,
        or until ``max_seconds`` / ``max_ticks``; ``t0`` is the stream time
        at which this run starts (for a restored server)."""
        torch = self.torch
        queue = sorted(list(self.queue) + list(requests), key=lambda r: r.arrival)
        self.queue = queue
        t_start = time.perf_counter() - t0
        ticks0 = self.ticks

        def now():
            return time.perf_counter() - t_start

        changed = bool(self.active)
        inflight = []
        while queue or self.active:
            t = now()
            if max_seconds is not None and t > max_seconds:
                break
            if max_ticks is not None and self.ticks - ticks0 >= max_ticks:
                break
            for r in [q for q in queue if q.arrival <= t or not realtime]:
                why = retire_reason(0, max(r.steps, 1), t - r.arrival, r.deadline,
                                    r.rid in self._cancel)
                if why in ("cancelled", "timed_out"):
                    queue.remove(r)
                    self._leave(r, why, t)
            while queue and (queue[0].arrival <= t or not realtime) and self._fits(queue[0]):
                r = queue.pop(0)
                r.admitted_at = t
                r.positions = torch.tensor(np.asarray(r.positions), device="cuda")
                r.velocities = torch.tensor(np.asarray(r.velocities), device="cuda")
                r.masses = torch.tensor(np.asarray(r.masses), device="cuda")
                r.acc = torch.zeros_like(r.positions)
                self.active.append(r)
                changed = True
            if not self.active:
                if queue and (queue[0].arrival <= t or not realtime):
                    # it does not fit even on an empty server: reject it
                    # rather than wait for room that never comes
                    self._leave(queue.pop(0), "rejected", t)
                elif queue and realtime:
                    time.sleep(max(0.0, min(queue[0].arrival - t, 0.05)))
                continue
            if changed:
                self._pack()
                changed = False
            self.tick()
            # the host runs at most two ticks ahead of the GPU: the next tick
            # is prepared while this one computes
            ev = torch.cuda.Event()
            ev.record()
            inflight.append(ev)
            if len(inflight) > 2:
                inflight.pop(0).synchronize()
            free, total = torch.cuda.mem_get_info()
            self.mem_peak = max(self.mem_peak, total - free)

            t = now()
            leaving = []
            for r in self.active:
                why = retire_reason(r.steps_done, r.steps, t - r.arrival, r.deadline,
                                    r.rid in self._cancel)
                if why:
                    leaving.append((r, why))
            if leaving:
                self._sync_roots()        # waits for the GPU; credits forced rebuilds
                t = now()
            for r, why in leaving:
                self.active.remove(r)
                self._leave(r, why, t)
            if leaving:
                changed = bool(self.active)
                if changed:
                    self._pack()          # drop the retired systems' state now
                    changed = False
                torch.cuda.empty_cache()  # and hand their blocks back
                _lib.check(self.L.bhut_pool_trim())
        torch.cuda.synchronize()
        wall = now() - t0
        self._sync_roots()
        solve_s = sum(a.elapsed_time(b) for a, b in self._solve_events) / 1e3
        self._solve_events = []
        done = [r for r in self.finished if r.status == "done"]
        lat = np.array([r.latency for r in done if r.latency is not None])
        by_class = latency_summary([(r.n, r.latency) for r in done if r.latency is not None])
        return {
            "requests_done": len(done),
            "requests_cancelled": sum(r.status == "cancelled" for r in self.finished),
            "requests_timed_out": sum(r.status == "timed_out" for r in self.finished),
            "requests_rejected": sum(r.status == "rejected" for r in self.finished),
            "wall_s": wall, "ticks": self.ticks,
            "solves": self.solves, "solves_per_s": self.solves / wall if wall else 0.0,
            "accels_per_s": self.accels / wall if wall else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else None,
            "latency_by_size": by_class,
            "requests_unfinished": len(self.active) + len(self.queue),
            "solve_budget": self.solve_budget,
            "peak_resident_bytes_est": self.peak_bytes,
            "device_mem_used_peak_bytes": self.mem_peak,
            "device_mem_request_peak_bytes": self.mem_peak - self.mem_base,
            "solve_device_s": solve_s,
            "solve_share_of_wall": solve_s / wall if wall else None,
        }

    # -- checkpoint / resume ----------------------------------------------------
    def snapshot(self) -> dict:
        """Host copy of every queued and resident request's state (call
        between ticks, e.g. after ``run(max_ticks=k)``)."""
        self.torch.cuda.synchronize()
        self._sync_roots()
        def host(x):
            return None if x is None else (x.cpu().numpy().copy() if hasattr(x, "cpu")
                                           else np.array(x, copy=True))
        reqs = []
        for r in self.active + self.queue:
            reqs.append({
                "rid": r.rid, "arrival": r.arrival, "steps": r.steps, "kind": r.kind,
                "deadline": r.deadline, "steps_done": r.steps_done, "solves": r.solves,
                "primed": r.primed, "admitted_at": r.admitted_at, "resident": r in self.active,
                "positions": host(r.positions), "velocities": host(r.velocities),
                "masses": host(r.masses), "acc": host(r.acc), "order": host(r.order),
                "root": None if r.root is None else np.array(r.root, copy=True),
                "forced_rebuilds": r.forced_rebuilds})
        return {"requests": reqs, "ticks": self.ticks, "solves": self.solves,
                "accels": self.accels, "cancelled": sorted(self._cancel)}

    def restore(self, snap: dict) -> list[Request]:
        """Loads a snapshot into this (fresh) server: resident requests are
        resident again in the same order, queued ones queued; returns the
        requests."""
        torch = self.torch
        out = []
        for d in snap["requests"]:
            r = Request(d["rid"], d["arrival"], d["positions"], d["velocities"], d["masses"],
                        steps=d["steps"], kind=d["kind"], deadline=d["deadline"])
            r.steps_done, r.solves, r.primed = d["steps_done"], d["solves"], d["primed"]
            r.admitted_at = d["admitted_at"]
            r.root, r.forced_rebuilds = d["root"], d["forced_rebuilds"]
            if d["resident"]:
                r.positions = torch.as_tensor(d["positions"], device="cuda")
                r.velocities = torch.as_tensor(d["velocities"], device="cuda")
                r.masses = torch.as_tensor(d["masses"], device="cuda")
                r.acc = torch.as_tensor(d["acc"], device="cuda")
                r.order = None if d["order"] is None else torch.as_tensor(d["order"],
                                                                          device="cuda")
                self.active.append(r)
            else:
                self.queue.append(r)
            out.append(r)
        self.ticks, self.solves, self.accels = snap["ticks"], snap["solves"], snap["accels"]
        self._cancel = set(snap["cancelled"])
        return out

    def close(self):
        self.solver.close()


def plain_path(requests: list[Request], *, theta: float = 0.5, softening: float = 0.01,
               G: float = 1.0, dt: float = 1e-3, rebuild_every: int = 10, form: str = "fast",
               leaf_size: int = 32, criterion: str = "bh", multipole: str = "mono",
               realtime: bool = True, max_seconds: float | None = None,
               order: str = "arrival") -> dict:
    """The same stream, one request at a time through the public Tree API.
    ``order``: "arrival" (first come, first served) or "shortest" (of the
    requests that have arrived, the one with the least work next -- the
    server's ordering, so that a comparison isolates batching and
    residency).  Stops starting requests after ``max_seconds``."""
    import torch
    pending = sorted(requests, key=lambda r: r.arrival)
    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    t_start = time.perf_counter()
    solves = 0
    accels = 0
    done = []
    while pending:
        t = time.perf_counter() - t_start
        if max_seconds is not None and t > max_seconds:
            break
        arrived = [r for r in pending if r.arrival <= t or not realtime]
        if not arrived:
            time.sleep(max(0.0, pending[0].arrival - t))
            continue
        if order == "shortest":
            r = min(arrived, key=lambda q: (q.n * q.steps, q.rid))
        else:
            r = arrived[0]
        pending = [q for q in pending if q is not r]
        x = torch.as_tensor(np.asarray(r.positions), device="cuda").clone()
        v = torch.as_tensor(np.asarray(r.velocities), device="cuda").clone()
        m = torch.as_tensor(np.asarray(r.masses), device="cuda").clone()
        tree = api.Tree(x, m, leaf_size=leaf_size, form=form, criterion=criterion,
                        multipole=multipole).build()
        a = tree.accelerations(theta=theta, softening=softening, G=G)
        solves += 1
        for step in range(r.steps):
            _leapfrog(L, x, v, a, r.n, 0.5 * dt, dt, stream)
            if (step + 1) % rebuild_every == 0:
                tree.rebuild(x, m)
            else:
                tree.refit(x, m)
            a = tree.accelerations(theta=theta, softening=softening, G=G)
            _leapfrog(L, x, v, a, r.n, 0.5 * dt, 0.0, stream)
            solves += 1
        torch.cuda.synchronize()
        accels += r.n * (r.steps + 1)
        r.final_positions, r.final_velocities = x.to("cpu"), v.to("cpu")
        r.status = "done"
        tree.close()
        r.done_at = time.perf_counter() - t_start
        done.append(r)
    wall = time.perf_counter() - t_start
    lat = np.array([r.done_at - r.arrival for r in done])
    return {"requests_done": len(done), "wall_s": wall, "solves": solves,
            "solves_per_s": solves / wall if wall else 0.0,
            "accels_per_s": accels / wall if wall else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else None,
            "latency_by_size": latency_summary([(r.n, r.done_at - r.arrival) for r in done]),
            "requests_unfinished": len(pending), "order": order,
            "config": {"form": form, "theta": theta, "criterion": criterion,
                       "multipole": multipole, "leaf_size": leaf_size}}


# ---------------------------------------------------------------------------
# The plain path's cost model (for stream-level comparisons)
# ---------------------------------------------------------------------------
def plain_service_times(requests: list[Request], *, theta: float = 0.5, softening: float = 0.01,
                        G: float = 1.0, dt: float = 1e-3, form: str = "fast",
                        leaf_size: int = 32, criterion: str = "bh",
                        multipole: str = "mono") -> list[dict]:
    """Measures what each request costs the plain per-request path (one
    ``Tree`` per request, as ``plain_path``): the initial solve (build +
    accelerations), one refit step and one rebuild step (half kick, drift,
    refit or rebuild, accelerations, half kick), each timed as host wall
    time with the device synchronised before and after.  The path runs one
    request at a time, so a request's cost does not depend on the others."""
    import torch
    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for r in requests:
        x = torch.as_tensor(np.asarray(r.positions), device="cuda").clone()
        v = torch.as_tensor(np.asarray(r.velocities), device="cuda").clone()
        m = torch.as_tensor(np.asarray(r.masses), device="cuda").clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tree = api.Tree(x, m, leaf_size=leaf_size, form=form, criterion=criterion,
                        multipole=multipole).build()
        a = tree.accelerations(theta=theta, softening=softening, G=G)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        times = []
        for rebuild in (False, True):
            _leapfrog(L, x, v, a, r.n, 0.5 * dt, dt, stream)
            if rebuild:
                tree.rebuild(x, m)
            else:
                tree.refit(x, m)
            a = tree.accelerations(theta=theta, softening=softening, G=G)
            _leapfrog(L, x, v, a, r.n, 0.5 * dt, 0.0, stream)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            times.append(t2 - t1)
            t1 = t2
        tree.close()
        out.append({"rid": r.rid, "n": r.n, "kind": r.kind, "t_prime": t1 - t0 - sum(times),
                    "t_refit": times[0], "t_rebuild": times[1]})
    return out


def request_cost(t: dict, steps: int, rebuild_every: int) -> float:
    """Plain-path seconds for one request of ``steps`` steps from its
    measured per-step costs (a rebuild every ``rebuild_every`` steps)."""
    rebuilds = steps // rebuild_every
    return t["t_prime"] + rebuilds * t["t_rebuild"] + (steps - rebuilds) * t["t_refit"]


def interpolate_service_times(measured: list[dict], requests: list[Request]) -> dict:
    """Per-request costs for every request: measured ones as they are, the
    others interpolated log-log in N between measured requests of the same
    kind (beyond the measured range: the nearest end, scaled in proportion
    to N above it).  Returns {rid: times}."""
    by_kind: dict[str, list[dict]] = {}
    for t in measured:
        by_kind.setdefault(t["kind"], []).append(t)
    known = {t["rid"]: t for t in measured}
    out = {}
    for r in requests:
        if r.rid in known:
            out[r.rid] = known[r.rid]
            continue
        pts = sorted(by_kind.get(r.kind) or measured, key=lambda t: t["n"])
        ln = np.log([t["n"] for t in pts])
        est = {"rid": r.rid, "n": r.n, "kind": r.kind, "interpolated": True}
        for key in ("t_prime", "t_refit", "t_rebuild"):
            lt = np.log([max(t[key], 1e-9) for t in pts])
            x = np.log(r.n)
            if x > ln[-1]:
                v = float(np.exp(lt[-1]) * r.n / pts[-1]["n"])
            else:
                v = float(np.exp(np.interp(x, ln, lt)))
            est[key] = v
        out[r.rid] = est
    return out


def simulate_sequential(requests: list[Request], costs: dict, *, steps: int,
                        rebuild_every: int, order: str = "shortest",
                        window: float | None = None) -> dict:
    """The plain path's schedule on a stream from per-request costs: one
    request at a time; when one finishes, the next is, of the requests that
    have arrived, the one with the least work (``order="shortest"``, the
    server's ordering) or the earliest.  ``window``: only what completes by
    then counts (a request in progress contributes the solves it finished).
    Returns the same summary fields as ``Server.run``."""
    pending = sorted(requests, key=lambda r: r.arrival)
    t = 0.0
    done = []
    solves = 0
    accels = 0
    while pending:
        if window is not None and t >= window:
            break
        arrived = [r for r in pending if r.arrival <= t]
        if not arrived:
            t = pending[0].arrival
            continue
        r = (min(arrived, key=lambda q: (q.n * q.steps, q.rid)) if order == "shortest"
             else arrived[0])
        pending.remove(r)
        c = costs[r.rid]
        dur = request_cost(c, steps, rebuild_every)
        if window is not None and t + dur > window:
            # partial: the initial solve, then whole steps at the mean step cost
            left = window - t - c["t_prime"]
            if left >= 0:
                per = dur - c["t_prime"]
                k = min(steps, int(left / (per / steps))) if per > 0 else steps
                solves += 1 + k
                accels += r.n * (1 + k)
            t = window
            break
        t += dur
        solves += steps + 1
        accels += r.n * (steps + 1)
        done.append((r, t))
    wall = t if window is None else window
    lat = [(r.n, end - r.arrival) for r, end in done]
    arr = np.array([x for _, x in lat])
    return {"requests_done": len(done), "wall_s": wall, "solves": solves,
            "solves_per_s": solves / wall if wall else 0.0,
            "accels_per_s": accels / wall if wall else 0.0,
            "latency_p50_s": float(np.percentile(arr, 50)) if arr.size else None,
            "latency_p99_s": float(np.percentile(arr, 99)) if arr.size else None,
            "latency_by_size": latency_summary(lat),
            "requests_unfinished": len(requests) - len(done), "order": order}
