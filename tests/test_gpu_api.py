"""Public-API behaviour on the GPU: input/output types, known answers and the
physics invariants the reference's own tests pin (tests/unit/test_api.py,
tests/unit/test_physics.py, tests/validation/test_physics_validation.py,
tests/edge_cases/test_boundary_conditions.py)."""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


def test_two_body_known_answer():
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    acc = bh.accelerations(pos, np.ones(2))
    assert acc.shape == (2, 3) and acc.dtype == np.float64
    np.testing.assert_allclose(np.linalg.norm(acc, axis=1), 1.0, rtol=1e-10)
    np.testing.assert_allclose(acc[0], -acc[1], rtol=1e-10)


def test_single_particle_zero():
    acc = bh.accelerations(np.zeros((1, 3)), np.ones(1))
    assert np.all(acc == 0.0)


def test_far_separation():
    pos = np.array([[0.0, 0, 0], [1e6, 0, 0]])
    acc = bh.accelerations(pos, np.ones(2))
    np.testing.assert_allclose(np.linalg.norm(acc, axis=1), 1e-12, rtol=1e-10)
    pos = np.array([[0.0, 0, 0], [1e15, 0, 0]])
    acc = bh.accelerations(pos, np.ones(2))
    assert np.all(np.isfinite(acc)) and np.all(np.linalg.norm(acc, axis=1) > 0)


def test_identical_positions_no_softening():
    pos = np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0], [0.0, 0.0, 0.0]])
    acc = bh.accelerations(pos, np.ones(3), softening=0.0)
    assert np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0], acc[1])


def test_G_linearity_and_newton3():
    pos, m = workloads.gaussian(500, seed=4)
    m = np.random.default_rng(1).uniform(0.5, 2, 500)
    a1 = bh.accelerations(pos, m, theta=0.0, softening=0.01)
    a2 = bh.accelerations(pos, m, theta=0.0, softening=0.01, G=2.0)
    np.testing.assert_allclose(a2, 2.0 * a1, rtol=1e-12)
    total = (m[:, None] * a1).sum(axis=0)
    assert np.all(np.abs(total) < 1e-12 * np.abs(m[:, None] * a1).sum())


def test_tree_matches_function_and_determinism():
    pos, m = workloads.plummer(20_000, seed=8)
    a = bh.accelerations(pos, m, theta=0.5, softening=0.01)
    t = bh.Tree(pos, m).build()
    b = t.accelerations(theta=0.5, softening=0.01)
    c = t.accelerations(theta=0.5, softening=0.01)
    assert np.array_equal(a, b) and np.array_equal(b, c)
    assert t._tree.mass[0] == pytest.approx(m.sum(), rel=1e-12)
    t.close()


def test_torch_cuda_in_cuda_out(oracle_mod):
    import torch
    pos, m = workloads.plummer(5000, seed=5)
    pd, md = torch.from_numpy(pos).cuda(), torch.from_numpy(m).cuda()
    acc = bh.accelerations(pd, md, theta=0.5, softening=0.01)
    assert isinstance(acc, torch.Tensor) and acc.is_cuda and acc.dtype == torch.float64
    ref = bh.accelerations(pos, m, theta=0.5, softening=0.01)
    assert np.array_equal(acc.cpu().numpy(), ref)
    # float32 tensors are promoted to float64, as np.asarray(dtype=float64)
    acc32 = bh.accelerations(pd.float(), md.float(), theta=0.5, softening=0.01)
    assert acc32.dtype == torch.float64
    tr = bh.Tree(pd, md).build()
    tg = torch.from_numpy(workloads.cube_targets(300, seed=1, side=3.0)).cuda()
    out = tr.accelerations(tg, theta=0.5, softening=0.01)
    assert out.is_cuda and tuple(out.shape) == (300, 3)
    tr.close()


def test_nonfinite_positions_rejected():
    pos = np.array([[0.0, 0, 0], [np.nan, 0, 0]])
    with pytest.raises(ValueError, match="finite"):
        bh.accelerations(pos, np.ones(2))


def test_refit_changes_result_and_rebuild_new_n():
    pos, m = workloads.gaussian(2000, seed=6)
    t = bh.Tree(pos, m, leaf_size=8).build()
    a0 = t.accelerations(theta=0.5, softening=0.01)
    pos2 = pos + 0.05 * np.random.default_rng(2).standard_normal(pos.shape)
    t.refit(pos2)
    a1 = t.accelerations(theta=0.5, softening=0.01)
    assert not np.allclose(a0, a1)
    # refit keeps stale geometry: compare against the oracle's refit
    from oracle import oracle
    ot = oracle.refit(oracle.build_tree(pos, m, 8), pos2, m)
    assert rel_l2(a1, oracle.accelerations(ot, pos2, m, theta=0.5, softening=0.01)) <= 1e-11
    pos3, m3 = workloads.gaussian(777, seed=7)
    t.rebuild(pos3, m3)
    assert t._tree.num_particles == 777
    a3 = t.accelerations(theta=0.5, softening=0.01)
    assert a3.shape == (777, 3)
    t.close()


def test_2d_and_leaf_sizes(oracle_mod):
    pos, m = workloads.gaussian(3000, seed=12, dim=2)
    for L in (1, 8, 33, 200):
        acc = bh.accelerations(pos, m, dim=2, leaf_size=L, theta=0.6, softening=0.02)
        ot = oracle_mod.build_tree(pos, m, L)
        ref = oracle_mod.accelerations(ot, pos, m, theta=0.6, softening=0.02)
        assert rel_l2(acc, ref) <= 1e-11, L


@pytest.mark.parametrize("form", ["exact", "fast", "fp32"])
def test_two_body_extremes(form, oracle_mod):
    """The reference's numerical edge cases (tests/edge_cases, two bodies,
    softening 0): coincident points, 1e-15 and 1e15 separations, 1e-15 and
    1e10 masses, 1e12 offsets with unit separation."""
    cases = [
        (np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0]]), np.array([1.0, 1.0])),
        (np.array([[0.0, 0.0, 0.0], [1e-15, 0.0, 0.0]]), np.array([1.0, 1.0])),
        (np.array([[0.0, 0.0, 0.0], [1e15, 0.0, 0.0]]), np.array([1.0, 1.0])),
        (np.array([[0.0, 0.0, 0.0], [1e6, 0.0, 0.0]]), np.array([1e-15, 1e-15])),
        (np.array([[0.0, 0.0, 0.0], [1e-6, 0.0, 0.0]]), np.array([1e10, 1e10])),
        (np.array([[1e12, 1e12, 1e12], [1e12 + 1.0, 1e12, 1e12]]), np.array([1.0, 1.0])),
    ]
    tol = {"exact": 1e-15, "fast": 1e-13, "fp32": 1e-6}[form]
    for pos, m in cases:
        acc = bh.accelerations(pos, m, form=form)
        ref = oracle_mod.accelerations(oracle_mod.build_tree(pos, m, 32), pos, m, theta=0.5,
                                       softening=0.0)
        assert np.all(np.isfinite(acc))
        assert np.allclose(acc, ref, rtol=tol, atol=0.0), (form, pos, acc, ref)
        assert np.allclose(acc[0], -acc[1] * m[1] / m[0], rtol=1e-12 if form != "fp32" else 1e-6)


def test_rejected_refit_leaves_tree_intact():
    """A refit with non-finite positions raises and the built tree still
    gives its previous accelerations (tests/integration/test_workflows.py:262-280
    in the reference checks the same for an invalid update)."""
    pos, m = workloads.gaussian(3000, seed=14)
    t = bh.Tree(pos, m, leaf_size=16).build()
    a0 = t.accelerations(theta=0.5, softening=0.01)
    bad = pos.copy()
    bad[17, 1] = np.nan
    with pytest.raises(ValueError, match="finite"):
        t.refit(bad)
    with pytest.raises(ValueError, match="finite"):
        t.rebuild(np.where(np.isnan(bad), np.inf, bad))
    a1 = t.accelerations(theta=0.5, softening=0.01)
    assert np.array_equal(a0, a1)
    t.close()


@pytest.mark.parametrize("form", ["exact", "fast"])
def test_physics_invariants(form):
    """Known answers and invariants of the reference's physics tests:
    regular tetrahedron (equal magnitudes, pointing at the centroid), inverse
    square, momentum sum, theta -> 0 against the direct sum, float32 inputs."""
    tet = np.array([[1.0, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    a = bh.accelerations(tet, np.ones(4), theta=0.0, form=form)
    mags = np.linalg.norm(a, axis=1)
    assert np.allclose(mags, mags[0], rtol=1e-12)
    unit_in = -tet / np.linalg.norm(tet, axis=1)[:, None]
    assert np.allclose(a / mags[:, None], unit_in, rtol=0, atol=1e-12)
    d1 = bh.accelerations(np.array([[0.0, 0, 0], [2.0, 0, 0]]), np.ones(2), form=form)
    d2 = bh.accelerations(np.array([[0.0, 0, 0], [4.0, 0, 0]]), np.ones(2), form=form)
    assert np.isclose(d1[0, 0] / d2[0, 0], 4.0, rtol=1e-12)
    pos, m = workloads.gaussian(500, seed=15)
    m = np.random.default_rng(1).uniform(0.5, 2.0, 500)
    a0 = bh.accelerations(pos, m, theta=0.0, softening=0.01, form=form)
    assert np.abs((m[:, None] * a0).sum(0)).max() < 1e-12 * np.abs(m[:, None] * a0).sum()
    direct = np.asarray(bh.direct_accelerations(pos, m, softening=0.01))
    a8 = bh.accelerations(pos, m, theta=1e-8, softening=0.01, form=form)
    assert rel_l2(a8, direct) < (1e-12 if form == "exact" else 1e-11)
    a32 = bh.accelerations(pos.astype(np.float32), m.astype(np.float32), theta=0.5,
                           softening=0.01, form=form)
    a64 = bh.accelerations(pos.astype(np.float32).astype(np.float64),
                           m.astype(np.float32).astype(np.float64), theta=0.5, softening=0.01,
                           form=form)
    assert np.array_equal(a32, a64) and a32.dtype == np.float64
