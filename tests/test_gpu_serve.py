"""Served form: continuous batching with device-resident leapfrog state."""
import numpy as np
import pytest

from bhut_gb300 import serve, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


def _req(rid, n, seed, steps=12, arrival=0.0):
    pos, m = workloads.plummer(n, seed=seed)
    vel = np.random.default_rng(seed).normal(0.0, 0.1, (n, 3))
    return serve.Request(rid, arrival, pos, vel, m, steps=steps)


def _run(reqs, **kw):
    sv = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=5, **kw)
    stats = sv.run(reqs, realtime=False)
    sv.close()
    return stats


def test_result_same_alone_and_in_the_mix():
    alone = _req(0, 3000, 1)
    st = _run([alone])
    assert st["requests_done"] == 1 and alone.solves == alone.steps + 1
    mix = [_req(0, 3000, 1), _req(1, 700, 2, steps=7), _req(2, 9000, 3, steps=20),
           _req(3, 150, 4, steps=3)]
    # a cap on resident particles forces admissions and retirements mid-run
    st = _run(mix, max_active_particles=10_000)
    assert st["requests_done"] == 4
    a = mix[0]
    assert np.array_equal(a.final_positions.cpu().numpy(), alone.final_positions.cpu().numpy())
    assert np.array_equal(a.final_velocities.cpu().numpy(),
                          alone.final_velocities.cpu().numpy())


def test_server_matches_plain_integration_within_tolerance():
    """The served FP32 trajectory stays within FP32 accuracy of the plain
    FP64-accurate per-request path with the same opening criterion."""
    r1 = _req(0, 4000, 5, steps=10)
    _run([r1], criterion="bh")
    r2 = _req(0, 4000, 5, steps=10)
    serve.plain_path([r2], theta=0.5, softening=0.01, dt=1e-3, rebuild_every=5,
                     realtime=False)
    # different arithmetic (FP32 + quadrupoles vs float-float monopoles) and
    # refit geometry: the trajectories differ by the Barnes-Hut truncation
    # error (~1e-3 of a) acting for 10 steps of dt=1e-3, far below the
    # distance the particles moved (~1e-3)
    assert r2.done_at is not None
    x1 = r1.final_positions.cpu().numpy()
    x2 = r2.final_positions.cpu().numpy()
    assert np.all(np.isfinite(x1))
    moved = np.linalg.norm(x2 - _req(0, 4000, 5).positions, axis=1).mean()
    diff = np.linalg.norm(x1 - x2, axis=1)
    assert diff.mean() < 1e-3 * moved and diff.max() < 0.2 * moved


def test_admission_budget():
    reqs = [_req(k, 2000, 10 + k, steps=2) for k in range(3)]
    sv = serve.Server(hbm_budget=2500 * serve.bytes_per_particle(16))
    st = sv.run(reqs, realtime=False)
    sv.close()
    assert st["requests_done"] == 3
    # never more than one system resident at a time under this budget
    assert st["peak_resident_bytes_est"] <= 2500 * serve.bytes_per_particle(16)


def test_cancel_and_deadline_leave_others_unchanged():
    alone = _req(0, 3000, 1)
    _run([alone])
    mix = [_req(0, 3000, 1), _req(1, 2000, 2, steps=50), _req(2, 1500, 3, steps=50),
           _req(3, 800, 4, steps=5)]
    mix[2].deadline = 0.0          # times out at the first tick boundary
    sv = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=5)
    sv.cancel(1)
    st = sv.run(mix, realtime=False)
    sv.close()
    assert [r.status for r in mix] == ["done", "cancelled", "timed_out", "done"]
    assert st["requests_done"] == 2 and st["requests_cancelled"] == 1
    assert st["requests_timed_out"] == 1 and st["device_mem_used_peak_bytes"] > 0
    assert np.array_equal(mix[0].final_positions.cpu().numpy(),
                          alone.final_positions.cpu().numpy())


def test_snapshot_restore_continues_bit_for_bit():
    ref = [_req(0, 3000, 1, steps=9), _req(1, 1200, 2, steps=14)]
    _run(ref)
    reqs = [_req(0, 3000, 1, steps=9), _req(1, 1200, 2, steps=14)]
    sv = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=5)
    sv.run(reqs, realtime=False, max_ticks=6)     # stop mid-run (a rebuild is due at 5)
    snap = sv.snapshot()
    sv.close()
    sv2 = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=5)
    back = sv2.restore(snap)
    sv2.run(realtime=False)
    sv2.close()
    for a, b in zip(sorted(back, key=lambda r: r.rid), ref):
        assert a.status == "done" and a.steps_done == b.steps_done
        assert np.array_equal(a.final_positions.cpu().numpy(), b.final_positions.cpu().numpy())
        assert np.array_equal(a.final_velocities.cpu().numpy(),
                              b.final_velocities.cpu().numpy())


def test_oversized_request_is_rejected_not_waited_for():
    reqs = [_req(0, 1500, 7, steps=2), _req(1, 6000, 8, steps=2)]
    sv = serve.Server(hbm_budget=3000 * serve.bytes_per_particle(16))
    st = sv.run(reqs, realtime=False, max_seconds=60)
    sv.close()
    assert [r.status for r in reqs] == ["done", "rejected"]
    assert st["requests_done"] == 1 and st["requests_rejected"] == 1


def test_refit_falls_back_to_rebuild_outside_root_box():
    """A system whose particles leave 1.1x the root box of its last rebuild is
    rebuilt (the reference's refit-vs-rebuild test), a quiet one is refitted;
    either way each trajectory is the same alone and in the mix."""
    def expanding():
        r = _req(0, 2000, 11, steps=6)
        r.velocities = 300.0 * r.positions          # +30 % per step of dt = 1e-3
        return r

    def quiet():
        return _req(1, 2500, 12, steps=6)
    alone = expanding()
    sv = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=100)
    sv.run([alone], realtime=False)
    sv.close()
    mix = [expanding(), quiet()]
    sv = serve.Server(theta=0.5, softening=0.01, dt=1e-3, rebuild_every=100)
    sv.run(mix, realtime=False)
    sv.close()
    assert alone.forced_rebuilds >= 4 and mix[0].forced_rebuilds == alone.forced_rebuilds
    assert mix[1].forced_rebuilds == 0
    assert np.array_equal(mix[0].final_positions.cpu().numpy(),
                          alone.final_positions.cpu().numpy())
