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
