"""Host logic of the served form: request stream, admission, refit/rebuild
schedule (no GPU)."""
import numpy as np

from bhut_gb300 import serve


def test_request_stream_is_seeded_and_shaped():
    a = serve.request_stream(12, rate=200.0, nmin=1000, nmax=20000, steps=5, seed=3)
    b = serve.request_stream(12, rate=200.0, nmin=1000, nmax=20000, steps=5, seed=3)
    assert [r.n for r in a] == [r.n for r in b]
    assert all(np.array_equal(x.positions, y.positions) for x, y in zip(a, b))
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and arr[0] > 0
    assert all(1000 <= r.n <= 20000 for r in a)
    assert {r.kind for r in a} <= {"plummer", "cube"}
    for r in a:
        assert r.positions.shape == (r.n, 3) and r.velocities.shape == (r.n, 3)
        assert np.isclose(r.masses.sum(), 1.0) and r.steps == 5
    v = np.concatenate([r.velocities for r in a])
    assert abs(v.std() - 0.1) < 0.01
    cubes = [r for r in a if r.kind == "cube"]
    if cubes:
        assert np.abs(cubes[0].positions).max() <= 1.0


def test_admission_budget_and_cap():
    bpp = serve.bytes_per_particle(16)
    budget = 10_000 * bpp
    assert serve.admits(0, 0, 10_000, leaf_size=16, hbm_budget=budget)
    assert not serve.admits(0, 0, 10_001, leaf_size=16, hbm_budget=budget)
    assert serve.admits(6_000, 1, 4_000, leaf_size=16, hbm_budget=budget)
    assert not serve.admits(6_000, 1, 4_001, leaf_size=16, hbm_budget=budget)
    # the particle cap: an empty server admits past it, a busy one does not
    assert serve.admits(0, 0, 5_000, leaf_size=16, hbm_budget=budget, max_active=1_000)
    assert not serve.admits(500, 1, 600, leaf_size=16, hbm_budget=budget, max_active=1_000)
    assert serve.admits(400, 1, 600, leaf_size=16, hbm_budget=budget, max_active=1_000)
    # smaller leaves hold more nodes per particle
    assert serve.bytes_per_particle(8) > serve.bytes_per_particle(32)


def test_refit_rebuild_schedule():
    # first solve of a request (not primed / no order): rebuild
    assert not serve.keeps_order(False, False, 0, 10)
    assert not serve.keeps_order(True, False, 3, 10)
    sched = [serve.keeps_order(True, True, s, 10) for s in range(25)]
    assert [s for s, k in enumerate(sched) if not k] == [0, 10, 20]


def test_retire_reasons():
    assert serve.retire_reason(3, 10, 0.5, None, False) is None
    assert serve.retire_reason(10, 10, 0.5, None, False) == "done"
    assert serve.retire_reason(3, 10, 0.5, 0.4, False) == "timed_out"
    assert serve.retire_reason(3, 10, 0.3, 0.4, False) is None
    # cancellation wins over everything, completion over the deadline
    assert serve.retire_reason(10, 10, 9.0, 0.4, True) == "cancelled"
    assert serve.retire_reason(10, 10, 9.0, 0.4, False) == "done"


def test_remaining_work_counts_the_initial_solve():
    assert serve.remaining_work(1000, 100, 0, False) == 1000 * 101
    assert serve.remaining_work(1000, 100, 0, True) == 1000 * 100
    assert serve.remaining_work(1000, 100, 100, True) == 0


def test_choose_running_shortest_work_first_within_budget():
    # (remaining work, particles, request id)
    work = [(5_000_000, 50_000, 0), (100_000, 1_000, 1), (900_000, 9_000, 2),
            (2_000_000_000, 2_000_000, 3), (300_000, 3_000, 4)]
    assert serve.choose_running(work, None) == [0, 1, 2, 3, 4]
    # budget 13,000 particles: ids 1, 4, 2 fit (13,000), 0 does not, 3 does not
    assert serve.choose_running(work, 13_000) == [1, 2, 4]
    # the shortest job always runs, even when larger than the budget
    assert serve.choose_running([(10**9, 2_000_000, 7)], 1000) == [0]
    # a later, smaller system fills the budget that a larger one skipped
    work2 = [(10, 10, 0), (20, 100, 1), (30, 5, 2)]
    assert serve.choose_running(work2, 20) == [0, 2]
    # ties broken by request id
    assert serve.choose_running([(7, 1, 9), (7, 1, 2)], 1) == [1]


def test_latency_summary_by_size_class():
    items = [(5_000, 1.0), (8_000, 3.0), (50_000, 10.0), (2_000_000, 100.0)]
    s = serve.latency_summary(items)
    assert s["all"]["count"] == 4
    assert s["n<1e4"]["count"] == 2 and s["n<1e4"]["p50_s"] == 2.0
    assert s["1e4<=n<1e5"]["p99_s"] == 10.0
    assert s["n>=1e5"]["count"] == 1
    assert serve.latency_summary([])["all"]["p50_s"] is None


def _req(rid, arrival, n, kind="plummer", steps=10):
    z = np.zeros((n, 3))
    return serve.Request(rid, arrival, z, z, np.ones(n), steps=steps, kind=kind)


def test_plain_request_cost_from_step_costs():
    t = {"t_prime": 1.0, "t_refit": 0.1, "t_rebuild": 0.3}
    assert np.isclose(serve.request_cost(t, 100, 10), 1.0 + 10 * 0.3 + 90 * 0.1)
    assert np.isclose(serve.request_cost(t, 10, 10), 1.0 + 0.3 + 9 * 0.1)


def test_service_time_interpolation():
    meas = [{"rid": 0, "n": 1000, "kind": "plummer", "t_prime": 1e-3, "t_refit": 1e-3,
             "t_rebuild": 2e-3},
            {"rid": 1, "n": 100_000, "kind": "plummer", "t_prime": 1e-1, "t_refit": 1e-1,
             "t_rebuild": 2e-1}]
    reqs = [_req(0, 0.0, 1000), _req(2, 0.0, 10_000), _req(3, 0.0, 200_000), _req(4, 0.0, 500)]
    c = serve.interpolate_service_times(meas, reqs)
    assert c[0] is meas[0]
    assert np.isclose(c[2]["t_refit"], 1e-2) and np.isclose(c[2]["t_rebuild"], 2e-2)
    assert np.isclose(c[3]["t_refit"], 2e-1)           # beyond: in proportion to N
    assert np.isclose(c[4]["t_refit"], 1e-3)           # below: the nearest end


def test_sequential_schedule_shortest_first_and_window():
    reqs = [_req(0, 0.0, 100), _req(1, 0.5, 100), _req(2, 0.6, 10)]
    costs = {0: {"t_prime": 0.0, "t_refit": 0.1, "t_rebuild": 0.1},
             1: {"t_prime": 0.0, "t_refit": 0.1, "t_rebuild": 0.1},
             2: {"t_prime": 0.0, "t_refit": 0.02, "t_rebuild": 0.02}}
    s = serve.simulate_sequential(reqs, costs, steps=10, rebuild_every=10, order="shortest")
    # r0 runs 0..1; then r2 (less work) 1..1.2; then r1 1.2..2.2
    assert s["requests_done"] == 3 and np.isclose(s["wall_s"], 2.2)
    assert s["solves"] == 33
    lat = sorted([1.0, 1.2 - 0.6, 2.2 - 0.5])
    assert np.isclose(s["latency_by_size"]["all"]["p50_s"], np.percentile(lat, 50))
    f = serve.simulate_sequential(reqs, costs, steps=10, rebuild_every=10, order="arrival")
    assert np.isclose(f["wall_s"], 2.2) and f["requests_done"] == 3
    w = serve.simulate_sequential(reqs, costs, steps=10, rebuild_every=10, order="shortest",
                                  window=1.1)
    # r0 done; r2 started at 1.0 and finished 5 of its 10 steps (plus its first solve)
    assert w["requests_done"] == 1 and w["solves"] == 11 + 1 + 5
    assert np.isclose(w["wall_s"], 1.1)
