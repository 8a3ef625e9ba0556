"""Batched form: many systems per solve, each result equal to solving that
system alone with the same form: bit for bit in form fp32; in form fast to
1e-12 (1.7e-14 measured), because a single-tree self solve of fewer targets than fill the GPU
gives each target 2-4 lanes (k_traverse_fast_lpt), which adds its pair terms
in another order than the batched kernel's one lane per target."""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import batch, workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


@pytest.fixture(scope="module")
def systems():
    return workloads.plummer_batch(nsys=40, nmin=64, nmax=6000, seed=3)


def _single(pos, m, form, theta=0.5, eps=0.01, leaf=32, multipole="mono"):
    t = bh.Tree(pos, m, leaf_size=leaf, form=form, multipole=multipole).build()
    a = t.accelerations(theta=theta, softening=eps)
    st = t._handle.stats()
    t.close()
    return a, st


@pytest.mark.parametrize("form,multipole", [("fast", "mono"), ("fp32", "mono"),
                                            ("fp32", "quad")])
def test_batch_equals_single_tree(systems, form, multipole):
    pos, m, off = batch.concat_systems(systems)
    sv = batch.BatchedSolver(form=form, targets_per_warp=32, use_graph=False,
                             multipole=multipole)
    sv.load(pos, m, off)
    acc = sv.solve(theta=0.5, softening=0.01)
    p2p_tot = 0
    for s, (p, mm) in enumerate(systems):
        ref, st = _single(p, mm, form, multipole=multipole)
        got = acc[off[s]:off[s + 1]]
        if form == "fp32":
            assert np.array_equal(got, ref), s
        else:
            assert rel_l2(got, ref) <= 1e-12, (s, rel_l2(got, ref))
        p2p_tot += st[0]
    assert sv.stats()[0] == p2p_tot
    sv.close()


@pytest.mark.parametrize("form,tol", [("fast", 1e-12), ("fp32", 1e-6)])
def test_batch_two_lanes_per_target(systems, form, tol):
    pos, m, off = batch.concat_systems(systems)
    a32 = batch.BatchedSolver(form=form, targets_per_warp=32, use_graph=False).load(
        pos, m, off).solve(theta=0.6, softening=0.02)
    sv = batch.BatchedSolver(form=form, targets_per_warp=16, use_graph=False)
    a16 = sv.load(pos, m, off).solve(theta=0.6, softening=0.02)
    assert rel_l2(a16, a32) < tol
    sv.close()


def test_graph_replay_and_reload(systems):
    import torch
    pos, m, off = batch.concat_systems(systems)
    pd, md = torch.from_numpy(pos).cuda(), torch.from_numpy(m).cuda()
    sv = batch.BatchedSolver(form="fp32", use_graph=True)
    sv.load(pd, md, off)
    out = torch.empty_like(pd)
    a1 = sv.solve(theta=0.5, softening=0.01, out=out).clone()
    a2 = sv.solve(theta=0.5, softening=0.01, out=out).clone()
    assert torch.equal(a1, a2)
    moved = pd * 1.01 + 0.001
    sv.load(moved, md, off)                 # same layout: the graph is replayed
    a3 = sv.solve(theta=0.5, softening=0.01, out=out).cpu().numpy()
    ref = batch.BatchedSolver(form="fp32", use_graph=False).load(
        moved.cpu().numpy(), m, off).solve(theta=0.5, softening=0.01)
    assert np.array_equal(a3, ref)
    sv.close()


def test_batch_fast_form_against_oracle(systems, oracle_mod):
    accs = batch.batched_accelerations(systems[:6], theta=0.5, softening=0.01, form="fast")
    for (p, mm), a in zip(systems[:6], accs):
        ot = oracle_mod.build_tree(p, mm, 32)
        ref = oracle_mod.accelerations(ot, p, mm, theta=0.5, softening=0.01)
        assert rel_l2(a, ref) <= 1e-11


def test_batch_2d_and_errors():
    sys2 = [workloads.gaussian(n, seed=n, dim=2) for n in (100, 700, 33)]
    accs = batch.batched_accelerations(sys2, theta=0.5, softening=0.02, form="fp32")
    for (p, mm), a in zip(sys2, accs):
        ref = bh.accelerations(p, mm, dim=2, form="fp32", theta=0.5, softening=0.02)
        assert np.array_equal(a, ref)
    with pytest.raises(ValueError):
        batch.BatchedSolver(form="exact")
    with pytest.raises(ValueError):
        batch.BatchedSolver(form="fast", criterion="bh_offset")


@pytest.mark.parametrize("form,tpw", [("fast", 32), ("fp32", 32), ("fp32", 16), ("fast", 16)])
def test_stack_placements_agree(systems, form, tpw):
    pos, m, off = batch.concat_systems(systems)
    res = {}
    for stk in ("shared", "registers"):
        sv = batch.BatchedSolver(form=form, targets_per_warp=tpw, use_graph=True, stack=stk)
        sv.load(pos, m, off)
        res[stk] = (sv.solve(theta=0.5, softening=0.01), sv.stats())
        sv.close()
    assert np.array_equal(res["shared"][0], res["registers"][0])
    assert res["shared"][1] == res["registers"][1]
    with pytest.raises(ValueError, match="stack must be"):
        batch.BatchedSolver(stack="global")


def test_batch_roots_and_outside_test():
    """The per-system refit-vs-rebuild test as a call: roots of the last
    solve, then flags for positions moved beyond 1.1x a root box."""
    import ctypes
    from bhut_gb300 import _lib
    L = _lib.load()
    systems = workloads.plummer_batch(nsys=3, nmin=500, nmax=2000, seed=9)
    pos, m, off = batch.concat_systems(systems)
    sv = batch.BatchedSolver(form="fp32", use_graph=False)
    sv.load(pos, m, off)
    sv.solve(theta=0.5, softening=0.01)
    roots = np.zeros((3, 4))
    _lib.check(L.bhut_batch_roots(sv.h, roots.ctypes.data))
    for s, (p, _) in enumerate(systems):
        lo, hi = p.min(0), p.max(0)
        assert np.all(roots[s, :3] >= lo) and np.all(roots[s, :3] <= hi)
        assert roots[s, 3] >= 0.5 * (hi - lo).max() * (1 - 1e-12)
    moved = pos.copy()
    moved[off[1]:off[2]] *= 3.0
    sv.load(moved, m, off)
    flags = np.zeros(3, dtype=np.uint8)
    _lib.check(L.bhut_batch_outside(sv.h, roots.ctypes.data, flags.ctypes.data))
    assert flags.tolist() == [0, 1, 0]
    used, reserved = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(L.bhut_pool_usage(ctypes.byref(used), ctypes.byref(reserved)))
    assert used.value > 0 and reserved.value >= used.value
    sv.close()
    _lib.check(L.bhut_pool_trim())
