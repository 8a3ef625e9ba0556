"""The FP32 precision form (FP32 traversal/P2P, Kahan-compensated sums) and
the offset opening criterion, on the GPU."""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import precision, workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


@pytest.fixture(scope="module")
def plummer200k():
    return workloads.plummer(200_000, seed=31)


def test_fp32_close_to_fp64_plain(plummer200k):
    pos, m = plummer200k
    t64 = bh.Tree(pos, m, form="fast").build()
    a64 = t64.accelerations(theta=0.5, softening=0.01)
    n64 = t64._handle.stats()
    t32 = bh.Tree(pos, m, form="fp32").build()
    a32 = t32.accelerations(theta=0.5, softening=0.01)
    n32 = t32._handle.stats()
    dist = precision.error_distribution(a32, a64)
    # FP32 arithmetic: ~1e-6 per target; an opening decision that flips at the
    # FP32/FP64 margin changes that target by the MAC error (~1e-3), rarely
    assert dist["median"] < 2e-6, dist
    assert dist["rel_l2"] < 1e-4, dist
    # the same interaction set up to decisions at the margin
    assert abs(n32[0] - n64[0]) <= 1e-4 * n64[0]
    assert abs(n32[1] - n64[1]) <= 1e-3 * n64[1]
    t64.close()
    t32.close()


def test_fp32_external_targets_and_2d():
    pos, m = workloads.gaussian(20_000, seed=3)
    tg = workloads.cube_targets(3000, seed=4, side=12.0)
    a = bh.Tree(pos, m, form="fp32").build().accelerations(tg, theta=0.6, softening=0.02)
    b = bh.Tree(pos, m, form="fast").build().accelerations(tg, theta=0.6, softening=0.02)
    assert rel_l2(a, b) < 1e-4
    pos2, m2 = workloads.gaussian(5000, seed=5, dim=2)
    a = bh.accelerations(pos2, m2, dim=2, form="fp32", theta=0.5, softening=0.02)
    b = bh.accelerations(pos2, m2, dim=2, form="fast", theta=0.5, softening=0.02)
    assert rel_l2(a, b) < 1e-4


def test_offset_criterion_is_more_accurate(plummer200k):
    pos, m = plummer200k
    idx = precision.sample_indices(len(pos), 1024, seed=2)
    ref = precision.direct_reference(pos, m, idx, softening=0.01)
    e_bh = precision.error_distribution(
        bh.accelerations(pos, m, form="fp32", theta=0.5, softening=0.01)[idx], ref)
    e_off = precision.error_distribution(
        bh.accelerations(pos, m, form="fp32", criterion="bh_offset", theta=0.5,
                         softening=0.01)[idx], ref)
    assert e_off["median"] < e_bh["median"]
    with pytest.raises(ValueError, match="form='fp32'"):
        bh.accelerations(pos[:10], m[:10], criterion="bh_offset", form="fast")


def test_direct_reference_matches_theta_zero():
    pos, m = workloads.plummer(4000, seed=8)
    idx = precision.sample_indices(len(pos), 256, seed=1)
    ref = precision.direct_reference(pos, m, idx, softening=0.01)
    a0 = bh.accelerations(pos, m, theta=0.0, softening=0.01, form="exact")
    assert rel_l2(a0[idx], ref) < 1e-13


def _quad_root_field(pos, m, tg, eps):
    """Monopole + traceless quadrupole of the whole cluster about its centre
    of mass, FP64, with r^2 -> r^2 + eps^2."""
    M = m.sum()
    com = (m[:, None] * pos).sum(0) / M
    s = pos - com
    Q = 3.0 * np.einsum("i,ij,ik->jk", m, s, s) - np.eye(3) * (m * (s * s).sum(1)).sum()
    d = com - tg
    r2 = (d * d).sum(1) + eps * eps
    Qd = d @ Q
    dQd = (d * Qd).sum(1)
    return (M / r2 ** 1.5 + 2.5 * dQd / r2 ** 3.5)[:, None] * d - Qd / r2[:, None] ** 2.5


def test_quadrupole_far_field_matches_expansion():
    # targets far from a flattened cluster: the root is accepted at once, so
    # the FP32 result is exactly the root's monopole + quadrupole
    pos, m = workloads.gaussian(3000, seed=12)
    pos = pos * np.array([1.0, 0.5, 0.2])
    rng = np.random.default_rng(5)
    tg = rng.normal(size=(500, 3))
    tg *= (60.0 / np.linalg.norm(tg, axis=1))[:, None]
    t = bh.Tree(pos, m, form="fp32", multipole="quad").build()
    a = t.accelerations(tg, theta=0.5, softening=0.05)
    assert t._handle.stats()[0] == 0            # no particle-particle pairs
    want = _quad_root_field(pos, m, tg, 0.05)
    assert rel_l2(a, want) < 1e-5
    exact = np.asarray(bh.direct_accelerations(pos, m, softening=0.05, targets=tg))
    mono = bh.Tree(pos, m, form="fp32").build().accelerations(tg, theta=0.5, softening=0.05)
    assert rel_l2(a, exact) < 0.1 * rel_l2(mono, exact)


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_quadrupoles_reduce_error(plummer200k, theta):
    pos, m = plummer200k
    idx = precision.sample_indices(len(pos), 1024, seed=2)
    ref = precision.direct_reference(pos, m, idx, softening=0.01)
    errs = {}
    for mp in ("mono", "quad"):
        a = bh.accelerations(pos, m, form="fp32", multipole=mp, theta=theta, softening=0.01)
        errs[mp] = precision.error_distribution(a[idx], ref)
    assert errs["quad"]["median"] < 0.4 * errs["mono"]["median"], errs
    # measured medians on this sample: theta 0.5: mono 2.7e-3 -> quad 5e-4;
    # theta 0.7: mono 6.5e-3 -> quad 1.3e-3
    assert errs["quad"]["median"] <= (1e-3 if theta <= 0.5 else 2e-3), errs
    # theta = 0 opens every node: no expansion is used, the forms agree
    small, sm = pos[:3000], m[:3000]
    a0 = bh.accelerations(small, sm, form="fp32", multipole="quad", theta=0.0, softening=0.01)
    b0 = bh.accelerations(small, sm, form="fp32", theta=0.0, softening=0.01)
    assert np.array_equal(a0, b0)
    with pytest.raises(ValueError, match="multipole must be 'mono'"):
        bh.accelerations(small, sm, form="fast", multipole="quad")


def test_results_carry_error_distributions():
    pos, m = workloads.plummer(20_000, seed=12)
    acc, dist = precision.accelerations_with_errors(pos, m, theta=0.5, softening=0.01,
                                                    multipole="quad", n_sample=512)
    assert acc.shape == pos.shape and dist["n"] == 512
    assert 0 < dist["median"] < 1e-3 and dist["median"] <= dist["p99"] <= dist["max"]
    systems = workloads.plummer_batch(4, 300, 3000, seed=2)
    out = precision.batched_with_errors(systems, theta=0.5, softening=0.01, n_sample=128)
    assert len(out) == 4
    for (p, _), (a, d) in zip(systems, out):
        assert a.shape == p.shape and d["n"] == min(128, len(p)) and d["median"] < 1e-2
