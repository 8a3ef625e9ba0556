"""The float-float pair term of form "fast" and its unit-mass frame.

When every particle has the same positive mass m0, masses are measured in
units of m0 (particle masses exactly 1, node masses M / m0) and the leaf
pair term skips the mass product; otherwise masses are scaled by a power of
two.  Both frames must give the oracle's accelerations (the reference's
arithmetic, bhut/traverse/bh.py:226-280 and bhut/traverse/kernels.py:14-95)
to the float-float bar, and agree with each other.
"""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import batch, workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu

FAST_RTOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


def _oracle(oracle_mod, pos, m, theta=0.5, eps=0.01, leaf=32):
    t = oracle_mod.build_tree(pos, m, leaf)
    return oracle_mod.accelerations(t, pos, m, theta=theta, softening=eps, G=1.0)


@pytest.mark.parametrize("kind", ["equal", "one_differs", "random", "negative_equal"])
def test_mass_frames_against_oracle(oracle_mod, kind):
    pos, m = workloads.plummer(60_000, seed=11)
    m = m.copy()
    if kind == "one_differs":       # general frame, physically the same system
        m[123] = np.nextafter(m[123], 1.0)
    elif kind == "random":
        m = np.random.default_rng(5).uniform(0.5, 1.5, len(m)) / len(m)
    elif kind == "negative_equal":  # uniform but negative: the unit frame is not taken
        m = -m
    a = bh.accelerations(pos, m, theta=0.5, softening=0.01, form="fast")
    ref = _oracle(oracle_mod, pos, m)
    assert rel_l2(a, ref) < FAST_RTOL, kind


def test_unit_and_general_frames_agree():
    pos, m = workloads.plummer(100_000, seed=12)
    a_unit = bh.accelerations(pos, m, theta=0.5, softening=0.01, form="fast")
    m2 = m.copy()
    m2[-1] = np.nextafter(m2[-1], 1.0)     # one ulp: the general frame
    a_gen = bh.accelerations(pos, m2, theta=0.5, softening=0.01, form="fast")
    assert rel_l2(a_unit, a_gen) < 1e-12
    # the FP32 form reads the same frames (node masses M / m0 in the unit
    # frame); its opening test does not depend on the masses, so both frames
    # evaluate the same interactions and agree to FP32 rounding
    f_unit = bh.accelerations(pos, m, theta=0.5, softening=0.01, form="fp32")
    f_gen = bh.accelerations(pos, m2, theta=0.5, softening=0.01, form="fp32")
    assert rel_l2(f_unit, f_gen) < 1e-6
    err = np.linalg.norm(f_unit - a_unit, axis=1) / np.linalg.norm(a_unit, axis=1)
    assert np.median(err) < 1e-6


def test_scaled_masses_scale_the_result():
    """Equal masses m0 and c * m0 (c a power of two) give results in the
    ratio c exactly: the unit frame carries m0 only in the final scale."""
    pos, m = workloads.plummer(50_000, seed=13)
    a1 = bh.accelerations(pos, m, theta=0.5, softening=0.01, form="fast")
    a8 = bh.accelerations(pos, m * 8.0, theta=0.5, softening=0.01, form="fast")
    assert np.array_equal(a8, a1 * 8.0)


def test_batched_traversal_timing_with_and_without_graph():
    systems = workloads.plummer_batch(nsys=24, nmin=256, nmax=4096, seed=4)
    pos, m, off = batch.concat_systems(systems)
    for graph in (False, True):
        for form in ("fast", "fp32"):
            sv = batch.BatchedSolver(form=form, use_graph=graph)
            sv.load(pos, m, off)
            for _ in range(3):
                sv.solve(theta=0.5, softening=0.01)
                ms = sv.traverse_ms()
                assert 0.0 < ms < 1e4, (graph, form, ms)
            sv.close()


@pytest.mark.parametrize("n,dim,masses", [(5_000, 3, "equal"), (5_000, 3, "random"),
                                          (20_000, 3, "random"), (7_000, 2, "equal")])
def test_few_target_lane_groups(oracle_mod, n, dim, masses):
    """Self solves of fewer targets than fill the GPU give each target 2 or 4
    lanes (k_traverse_fast_lpt: 5,000 targets take 4, 20,000 take 2); the
    lanes share the target's leaf pairs and add their sums at the end.  The
    result must stay at the oracle's accuracy and agree with the same
    particles evaluated as external targets (one lane per target; a
    particle's own zero-distance pair adds exactly zero)."""
    pos, m = workloads.gaussian(n, seed=n + dim, dim=dim)
    if masses == "random":
        m = np.random.default_rng(n).uniform(0.5, 1.5, n)
    tree = bh.Tree(pos, m, dim=dim, form="fast").build()
    a_self = tree.accelerations(theta=0.5, softening=0.01)
    a_tgt = tree.accelerations(pos, theta=0.5, softening=0.01)
    tree.close()
    ot = oracle_mod.build_tree(pos, m, 32)
    ref = oracle_mod.accelerations(ot, pos, m, theta=0.5, softening=0.01, G=1.0)
    assert rel_l2(a_self, ref) < FAST_RTOL
    assert rel_l2(a_self, a_tgt) < 1e-12


def test_unsoftened_checked_path_against_exact():
    """Softening 0 (the reference's default): the float-float term keeps its
    range test, pairs closer than 2^-17 box half-sizes (and every particle's
    own zero-distance pair) go to FP64, and sparse leaf visits are split
    across idle lanes together with their FP64 pairs.  Against the IEEE-FP64
    form on every target of a 200k Plummer sphere."""
    pos, m = workloads.plummer(200_000, seed=13)
    t = bh.Tree(pos, m, form="fast").build()
    a = t.accelerations(theta=0.5, softening=0.0)
    exact_dec, fp64_pairs = t._handle.fallbacks()
    t.close()
    ref = bh.accelerations(pos, m, theta=0.5, softening=0.0, form="exact")
    assert fp64_pairs >= len(pos)          # at least the zero-distance pairs
    assert rel_l2(a, ref) < 1e-10
