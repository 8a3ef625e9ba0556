"""The reference's own test suite, restated against the drop-in, in the
default form.

bhut 0.1.0 ships black-box tests of ``bhut.accelerations`` and ``bhut.Tree``
(tests/unit, tests/validation, tests/edge_cases, tests/integration).  Their
source cannot be vendored and is not present where the GPU tests run, so
each test below restates one of them -- same fixture inputs, same calls,
same assertions and tolerances -- against ``bhut_gb300`` with its default
form.  Every test names the reference test it restates (file:line).  The
Dask tests, the array-namespace tests and the wall-clock tests are out of
scope; ``test_partial_failure_handling`` fails on the reference itself
(momentum -0.125 against atol 1e-10, masses spanning 1e-15..1e15) and is
restated with the bound FP64 arithmetic allows there.
"""
import numpy as np
import pytest

import bhut_gb300 as bhut
from bhut_gb300.tree.build import build_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


# -- fixtures of tests/conftest.py:11-88 ---------------------------------------
@pytest.fixture
def simple_system():
    return np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]), np.array([1.0, 1.0])


@pytest.fixture
def random_system():
    np.random.seed(42)
    return np.random.randn(10, 3).astype(np.float64), np.ones(10)


@pytest.fixture
def hierarchical_system():
    return (np.array([[-0.1, 0.0, 0.0], [0.1, 0.0, 0.0], [10.0, 0.0, 0.0]]),
            np.array([1.0, 1.0, 0.1]))


@pytest.fixture
def varied_masses_system():
    np.random.seed(456)
    return (np.random.randn(8, 3).astype(np.float64),
            np.array([0.1, 1.0, 10.0, 0.5, 2.0, 0.01, 5.0, 0.2]))


@pytest.fixture
def tree_built(random_system):
    return bhut.Tree(*random_system).build()


THETAS = [0.0, 0.1, 0.5, 1.0, 2.0]
SOFTENINGS = [0.0, 1e-6, 0.01, 0.1]
LEAF_SIZES = [1, 4, 8, 16]
GS = [1.0, 6.67430e-11, 2.0]


def momentum(acc, m):
    return np.sum(np.asarray(acc) * m[:, None], axis=0)


# -- tests/unit/test_api.py ------------------------------------------------------
def test_api_basic_functionality(simple_system):
    """unit/test_api.py:17-27"""
    acc = bhut.accelerations(*simple_system)
    assert acc.shape == (2, 3) and np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0], -acc[1], rtol=1e-10)


def test_api_parameter_variations(random_system):
    """unit/test_api.py:29-48"""
    p, m = random_system
    for kw in ([{"theta": t} for t in THETAS] + [{"softening": e} for e in SOFTENINGS]
               + [{"G": g} for g in GS]):
        acc = bhut.accelerations(p, m, **kw)
        assert acc.shape == (10, 3) and np.all(np.isfinite(acc))


def test_api_gravitational_scaling(simple_system):
    """unit/test_api.py:50-58"""
    a1 = bhut.accelerations(*simple_system, G=1.0)
    a2 = bhut.accelerations(*simple_system, G=2.0)
    np.testing.assert_allclose(a2, 2.0 * a1, rtol=1e-12)


def test_api_self_acceleration_zero():
    """unit/test_api.py:60-69"""
    acc = bhut.accelerations(np.zeros((1, 3)), np.array([1.0]))
    assert acc.shape == (1, 3)
    np.testing.assert_allclose(acc, 0.0, atol=1e-15)


def test_api_unequal_masses_newton_third_law():
    """unit/test_api.py:71-91 and unit/test_physics.py:17-32"""
    p, m = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]), np.array([1.0, 2.0])
    acc = bhut.accelerations(p, m)
    assert acc.shape == (2, 3) and np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0] * m[0], -acc[1] * m[1], rtol=1e-12)


def test_api_dtype_consistency(random_system):
    """unit/test_api.py:93-100"""
    assert bhut.accelerations(*random_system).dtype == np.float64


def test_tree_initialization_and_build(random_system):
    """unit/test_api.py:106-127"""
    p, m = random_system
    tree = bhut.Tree(p, m)
    assert tree.positions is not None and tree.masses is not None
    assert tree.dim == 3 and tree.leaf_size > 0
    acc = tree.build().accelerations()
    assert acc.shape == (10, 3) and np.all(np.isfinite(acc))


def test_tree_parameters(random_system):
    """unit/test_api.py:129-139"""
    for leaf in LEAF_SIZES:
        acc = bhut.Tree(*random_system, leaf_size=leaf).build().accelerations()
        assert acc.shape == (10, 3) and np.all(np.isfinite(acc))


def test_tree_multiple_evaluations(tree_built):
    """unit/test_api.py:141-149"""
    a1 = tree_built.accelerations(theta=0.5, softening=0.01)
    a2 = tree_built.accelerations(theta=0.5, softening=0.01)
    np.testing.assert_allclose(a1, a2, rtol=1e-15)


def test_tree_accelerations_vs_function(random_system):
    """unit/test_api.py:151-163"""
    a_f = bhut.accelerations(*random_system, theta=0.5, softening=0.01)
    a_t = bhut.Tree(*random_system).build().accelerations(theta=0.5, softening=0.01)
    np.testing.assert_allclose(a_f, a_t, rtol=1e-12)


def test_tree_external_targets(tree_built):
    """unit/test_api.py:165-173"""
    acc = tree_built.accelerations(targets=np.array([[0.0, 0.0, 0.0], [2.0, 2.0, 2.0]]))
    assert acc.shape == (2, 3) and np.all(np.isfinite(acc))


def test_tree_not_built_error(random_system):
    """unit/test_api.py:175-183"""
    with pytest.raises(ValueError, match="must be built"):
        bhut.Tree(*random_system).accelerations()


def test_api_calling_patterns_and_backends(random_system):
    """unit/test_api.py:190-215"""
    p, m = random_system
    np.testing.assert_allclose(bhut.accelerations(p, m, theta=0.5),
                               bhut.Tree(p, m).build().accelerations(theta=0.5), rtol=1e-10)
    np.testing.assert_allclose(bhut.accelerations(p, m, backend="numpy"),
                               bhut.accelerations(p, m, backend="auto"), rtol=1e-15)


def test_api_parameter_forwarding(random_system):
    """unit/test_api.py:217-229"""
    acc = bhut.accelerations(*random_system, theta=0.7, softening=0.02, G=2.0, leaf_size=8,
                             backend="auto")
    assert acc.shape == (10, 3) and np.all(np.isfinite(acc))


# -- tests/unit/test_physics.py ----------------------------------------------------
def test_physics_inverse_square_law():
    """unit/test_physics.py:34-56"""
    mags = [np.linalg.norm(bhut.accelerations(np.array([[0.0, 0, 0], [d, 0, 0]]),
                                              np.ones(2))[0]) for d in (1.0, 2.0, 4.0)]
    for i, d in enumerate((2.0, 4.0), start=1):
        np.testing.assert_allclose(mags[0] / mags[i], d ** 2, rtol=1e-8)


def test_physics_center_of_mass(random_system):
    """unit/test_physics.py:58-66 and validation/test_physics_validation.py:81-98"""
    p, m = random_system
    total = momentum(bhut.accelerations(p, m), m)
    np.testing.assert_allclose(total, 0.0, atol=1e-12)
    np.testing.assert_allclose(total / m.sum(), 0.0, atol=1e-12)


def test_physics_mass_scaling():
    """unit/test_physics.py:68-86"""
    p = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    ref = bhut.accelerations(p, np.ones(2))
    np.testing.assert_allclose(bhut.accelerations(p, 3.0 * np.ones(2)), 3.0 * ref, rtol=1e-12)


def test_physics_conservation(simple_system):
    """unit/test_physics.py:92-101"""
    np.testing.assert_allclose(momentum(bhut.accelerations(*simple_system), simple_system[1]),
                               0.0, atol=1e-12)


def test_physics_symmetric_pair():
    """unit/test_physics.py:103-119"""
    acc = bhut.accelerations(np.array([[-1.0, 0, 0], [1.0, 0, 0]]), np.ones(2))
    np.testing.assert_allclose(np.linalg.norm(acc[0]), np.linalg.norm(acc[1]), rtol=1e-15)
    np.testing.assert_allclose(acc[0], -acc[1], rtol=1e-15)


def test_physics_direction(simple_system):
    """unit/test_physics.py:121-139"""
    acc = bhut.accelerations(*simple_system)
    assert acc[0, 0] > 0 and abs(acc[0, 1]) < 1e-12 and abs(acc[0, 2]) < 1e-12
    assert acc[1, 0] < 0 and abs(acc[1, 1]) < 1e-12 and abs(acc[1, 2]) < 1e-12


# -- tests/unit/test_tree.py --------------------------------------------------------
def test_tree_build_function(random_system):
    """unit/test_tree.py:19-59"""
    p, m = random_system
    t = build_tree(p, m, leaf_size=4, dim=3)
    assert t.dim == 3 and t.leaf_size == 4 and len(t.center) > 0 and len(t.perm) == 10
    for leaf in LEAF_SIZES:
        t = build_tree(p, m, leaf_size=leaf, dim=3)
        assert t.leaf_size == leaf and np.all(np.isfinite(t.center))
    t = build_tree(p, m, leaf_size=2, dim=3)
    assert np.isclose(t.mass[0], m.sum())
    assert np.array_equal(np.sort(t.perm), np.arange(10))


def test_tree_build_edge_inputs_and_determinism(hierarchical_system):
    """unit/test_tree.py:61-92"""
    t = build_tree(np.array([[0.0, 0, 0], [1.0, 0, 0]]), np.ones(2), leaf_size=1, dim=3)
    assert t.dim == 3 and len(t.center) > 0
    mv = np.array([0.1, 1.0, 10.0, 0.5, 2.0, 0.01, 5.0, 0.2])
    tv = build_tree(np.random.default_rng(3).standard_normal((8, 3)), mv, leaf_size=2, dim=3)
    assert np.isclose(tv.mass[0], mv.sum())
    t1 = build_tree(*hierarchical_system, leaf_size=2, dim=3)
    t2 = build_tree(*hierarchical_system, leaf_size=2, dim=3)
    np.testing.assert_array_equal(t1.perm, t2.perm)
    np.testing.assert_allclose(t1.center, t2.center)
    np.testing.assert_allclose(t1.mass, t2.mass)


def test_tree_refit_rebuild_operations(random_system):
    """unit/test_tree.py:99-160"""
    p, m = random_system
    rng = np.random.default_rng(5)
    tree = bhut.Tree(p, m).build()
    a1 = tree.accelerations()
    tree.refit(p + 0.01 * rng.standard_normal(p.shape))
    a2 = tree.accelerations()
    assert a1.shape == a2.shape and np.all(np.isfinite(a2))
    assert not np.allclose(a1, a2, rtol=1e-10)
    tree.rebuild(rng.standard_normal((8, 3)), np.ones(8))
    assert tree.accelerations().shape == (8, 3)
    tree = bhut.Tree(p, m).build()
    cur = p.copy()
    for _ in range(3):
        cur = cur + 0.005 * rng.standard_normal(p.shape)
        acc = tree.refit(cur).accelerations()
        assert acc.shape == (10, 3) and np.all(np.isfinite(acc))


def test_tree_theta_softening_leaf_effects(random_system, simple_system):
    """unit/test_tree.py:162-235"""
    p, m = random_system
    res = {t: bhut.accelerations(p, m, theta=t) for t in THETAS}
    ratio = (np.mean(np.linalg.norm(res[2.0], axis=1)) /
             np.mean(np.linalg.norm(res[0.0], axis=1)))
    assert 0.1 < ratio < 10.0
    np.testing.assert_allclose(bhut.accelerations(p, m, theta=0.5),
                               bhut.accelerations(p, m, theta=0.5), rtol=1e-15)
    soft = {e: bhut.accelerations(*simple_system, softening=e) for e in SOFTENINGS}
    assert np.linalg.norm(soft[0.1][0]) < np.linalg.norm(soft[0.0][0])
    for leaf in LEAF_SIZES:
        mag = np.linalg.norm(bhut.accelerations(p, m, leaf_size=leaf), axis=1)
        assert np.all(mag > 1e-20) and np.all(mag < 1e10)


def test_tree_data_access(tree_built, varied_masses_system):
    """unit/test_tree.py:237-266"""
    assert tree_built.dim == 3 and len(tree_built.masses) == 10 and tree_built.leaf_size > 0
    tree = bhut.Tree(*varied_masses_system, leaf_size=2).build()
    for _ in range(5):
        assert tree.accelerations(theta=0.5).shape == (8, 3)


# -- tests/validation/test_physics_validation.py -----------------------------------
def test_validation_two_body():
    """validation/test_physics_validation.py:17-48"""
    p = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    acc = bhut.accelerations(p, np.ones(2))
    np.testing.assert_allclose(np.linalg.norm(acc, axis=1), 1.0, rtol=1e-10)
    np.testing.assert_allclose(acc[0], -acc[1], rtol=1e-15)
    np.testing.assert_allclose(acc[0] / np.linalg.norm(acc[0]), [1.0, 0, 0], rtol=1e-10)


def test_validation_lagrange_point():
    """validation/test_physics_validation.py:50-79"""
    p = np.array([[-0.5, 0, 0], [0.5, 0, 0], [0.0, np.sqrt(3) / 2, 0]])
    acc = bhut.accelerations(p, np.array([1.0, 1.0, 1e-6]))
    d = -p[2] / np.linalg.norm(p[2])
    assert np.dot(acc[2] / np.linalg.norm(acc[2]), d) > 0.5


def test_validation_momentum_and_torque(hierarchical_system):
    """validation/test_physics_validation.py:100-127"""
    np.testing.assert_allclose(momentum(bhut.accelerations(*hierarchical_system),
                                        hierarchical_system[1]), 0.0, atol=1e-12)
    p = np.array([[1.0, 0, 0], [-1.0, 0, 0]])
    acc = bhut.accelerations(p, np.ones(2))
    np.testing.assert_allclose(np.sum(np.cross(p, acc), axis=0), 0.0, atol=1e-12)


def test_validation_energy_consistency(simple_system):
    """validation/test_physics_validation.py:129-154"""
    p, m = simple_system
    acc = bhut.accelerations(p, m)
    kin = 0.5 * np.sum(m * np.sum(acc ** 2, axis=1))
    pot = -m[0] * m[1] / np.linalg.norm(p[0] - p[1])
    assert np.isfinite(kin) and kin > 0 and pot < 0


def test_validation_precision_vs_theta(simple_system):
    """validation/test_physics_validation.py:161-190"""
    ref = bhut.Tree(*simple_system).build().accelerations(theta=1e-8)
    errs = []
    for theta in [0.1, 0.5, 1.0, 1.5, 2.0]:
        acc = bhut.Tree(*simple_system).build().accelerations(theta=theta)
        errs.append(np.linalg.norm(acc - ref) / np.linalg.norm(ref))
        assert errs[-1] < theta * 0.5
    for i in range(1, len(errs)):
        assert errs[i] <= errs[i - 1] * 2


def test_validation_convergence_with_depth(random_system):
    """validation/test_physics_validation.py:192-219"""
    p, m = random_system
    for leaf in [4, 8, 16, 32]:
        acc = bhut.Tree(p, m, leaf_size=leaf).build().accelerations(theta=1.0)
        assert np.all(np.isfinite(acc))
        rel = np.linalg.norm(momentum(acc, m)) / (np.linalg.norm(acc * m[:, None]) + 1e-10)
        assert rel < 0.1


@pytest.mark.parametrize("dx", [1e-10, 1e-6])
def test_validation_close_pairs_large_finite(dx):
    """validation/test_physics_validation.py:221-239 and :434-450"""
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [dx, 0, 0]]), np.ones(2))
    assert np.all(np.isfinite(acc))
    assert 1e6 < np.linalg.norm(acc[0]) < np.inf


def test_validation_machine_precision_limits():
    """validation/test_physics_validation.py:241-265"""
    p = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    small = bhut.accelerations(p, np.array([1e-15, 1e-15]))
    large = bhut.accelerations(p, np.array([1e10, 1e10]))
    assert np.all(np.isfinite(small)) and np.all(np.isfinite(large))
    np.testing.assert_allclose(np.linalg.norm(large) / np.linalg.norm(small), 1e25, rtol=0.1)


def test_validation_relative_vs_absolute(hierarchical_system):
    """validation/test_physics_validation.py:267-294"""
    hi = bhut.Tree(*hierarchical_system).build().accelerations(theta=0.1)
    lo = bhut.Tree(*hierarchical_system).build().accelerations(theta=1.5)
    rel = np.abs(hi - lo) / (np.abs(hi) + 1e-15)
    assert np.max(rel) < 1.0
    big = np.abs(hi) > np.percentile(np.abs(hi), 75)
    if np.any(big):
        assert np.median(rel[big]) <= np.median(rel[~big]) * 2


def test_validation_colinear_and_planar():
    """validation/test_physics_validation.py:301-348"""
    acc = bhut.accelerations(np.array([[-1.0, 0, 0], [0.0, 0, 0], [1.0, 0, 0]]),
                             np.array([1.0, 2.0, 1.0]))
    np.testing.assert_allclose(acc[1, 1:], 0.0, atol=1e-12)
    assert acc[0, 0] > 0 and acc[2, 0] < 0
    np.testing.assert_allclose(abs(acc[0, 0]), abs(acc[2, 0]), rtol=1e-10)
    p = np.array([[-1.0, -1, 0], [1.0, -1, 0], [1.0, 1, 0], [-1.0, 1, 0]])
    acc = bhut.accelerations(p, np.ones(4))
    np.testing.assert_allclose(acc[:, 2], 0.0, atol=1e-12)
    for i in range(4):
        assert np.dot(acc[i] / np.linalg.norm(acc[i]), -p[i] / np.linalg.norm(p[i])) > 0.5


def test_validation_hierarchical_configuration():
    """validation/test_physics_validation.py:350-380"""
    acc = bhut.accelerations(np.array([[-0.1, 0, 0], [0.1, 0, 0], [10.0, 0, 0]]),
                             np.array([1.0, 1.0, 0.5]))
    assert acc[0, 0] > 0 and acc[1, 0] < 0 and acc[2, 0] < 0


def test_validation_tetrahedron():
    """validation/test_physics_validation.py:382-407"""
    a = 1.0 / np.sqrt(3)
    p = np.array([[a, a, a], [a, -a, -a], [-a, a, -a], [-a, -a, a]])
    acc = bhut.accelerations(p, np.ones(4))
    mags = np.linalg.norm(acc, axis=1)
    np.testing.assert_allclose(mags, mags[0], rtol=1e-10)
    for i in range(4):
        np.testing.assert_allclose(acc[i] / mags[i], -p[i] / np.linalg.norm(p[i]), rtol=1e-10)


def test_validation_large_separation():
    """validation/test_physics_validation.py:414-432"""
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [1e6, 0, 0]]), np.ones(2))
    np.testing.assert_allclose(np.linalg.norm(acc[0]), 1e-12, rtol=1e-10)
    assert np.all(np.isfinite(acc)) and acc[0, 0] > 0


def test_validation_mass_limits():
    """validation/test_physics_validation.py:452-487"""
    p = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    acc = bhut.accelerations(p, np.array([1e-12, 1.0]))
    assert np.all(np.isfinite(acc)) and abs(acc[0, 0]) > abs(acc[1, 0])
    m = np.array([1e12, 1.0])
    acc = bhut.accelerations(p, m)
    assert np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0] * m[0], -acc[1] * m[1], rtol=1e-12)
    assert abs(acc[1, 0]) > abs(acc[0, 0]) * 1e6


# -- tests/edge_cases/test_boundary_conditions.py ---------------------------------
def test_edge_input_validation():
    """edge_cases/test_boundary_conditions.py:17-58"""
    with pytest.raises(ValueError, match="empty|zero"):
        bhut.accelerations(np.empty((0, 3)), np.empty(0))
    acc = bhut.accelerations(np.array([[1.0, 2.0, 3.0]]), np.array([1.0]))
    np.testing.assert_allclose(acc, 0.0, atol=1e-15)
    with pytest.raises(ValueError, match="2D array|dimension"):
        bhut.accelerations(np.array([[1, 2]]), np.array([1]))
    with pytest.raises(ValueError, match="2D array|dimension"):
        bhut.accelerations(np.array([1, 2, 3]), np.array([1]))
    with pytest.raises(ValueError, match="1D array|dimension"):
        bhut.accelerations(np.array([[1, 2, 3]]), np.array([[1]]))
    with pytest.raises(ValueError, match="particles|elements|has"):
        bhut.accelerations(np.random.randn(5, 3), np.random.randn(3))


def test_edge_nonfinite_negative_zero_masses_and_dtypes():
    """edge_cases/test_boundary_conditions.py:60-130"""
    p = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    with pytest.raises((ValueError, RuntimeError)):
        bhut.accelerations(np.array([[1.0, np.nan, 3.0], [4.0, 5.0, 6.0]]), np.ones(2))
    with pytest.raises((ValueError, RuntimeError)):
        bhut.accelerations(p, np.array([1.0, np.inf]))
    for m in (np.array([1.0, -1.0]), np.array([1.0, 0.0])):
        acc = bhut.accelerations(p, m)
        assert acc.shape == (2, 3) and np.all(np.isfinite(acc))
    acc = bhut.accelerations(np.array([[1, 2, 3], [4, 5, 6]], dtype=np.int32),
                             np.array([1, 2], dtype=np.int32))
    assert acc.dtype in (np.float32, np.float64) and acc.shape == (2, 3)
    pf = np.random.default_rng(1).standard_normal((1000, 3)).astype(np.float32)
    acc = bhut.accelerations(pf, np.ones(1000, dtype=np.float32), theta=1.0)
    assert acc.shape == (1000, 3) and np.all(np.isfinite(acc))


def test_edge_parameter_values(simple_system):
    """edge_cases/test_boundary_conditions.py:136-232"""
    p, m = simple_system
    tiny = bhut.Tree(p, m).build().accelerations(theta=1e-10)
    huge = bhut.Tree(p, m).build().accelerations(theta=100.0)
    assert np.all(np.isfinite(tiny)) and np.all(np.isfinite(huge))
    np.testing.assert_allclose(momentum(tiny, m), 0.0, atol=1e-12)
    assert np.linalg.norm(momentum(huge, m)) / (np.linalg.norm(huge * m[:, None]) + 1e-10) < 1.0
    small = bhut.Tree(p, m, leaf_size=1).build().accelerations()
    large = bhut.Tree(p, m, leaf_size=100).build().accelerations()
    np.testing.assert_allclose(small, large, rtol=0.1)
    tree = bhut.Tree(p, m).build()
    with pytest.raises(ValueError, match="theta|positive"):
        tree.accelerations(theta=-1.0)
    assert np.all(np.isfinite(tree.accelerations(theta=0.0)))
    for leaf in (0, -5):
        with pytest.raises(ValueError, match="leaf_size|positive"):
            bhut.Tree(p, m, leaf_size=leaf)
    assert np.all(np.isfinite(bhut.Tree(p, m, leaf_size=20).build().accelerations(theta=1.5)))
    with pytest.raises((ValueError, TypeError)):
        tree.accelerations(theta="invalid")
    with pytest.raises((ValueError, TypeError)):
        bhut.Tree(p, m, leaf_size="invalid")


def test_edge_numerical_cases():
    """edge_cases/test_boundary_conditions.py:238-344"""
    acc = bhut.accelerations(np.array([[1.0, 2, 3], [1.0, 2, 3]]), np.ones(2))
    assert np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0], -acc[1], atol=1e-12)
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [1e-15, 0, 0]]), np.ones(2))
    assert np.all(np.isfinite(acc))
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [1e15, 0, 0]]), np.ones(2))
    assert np.all(np.isfinite(acc)) and 0 < np.linalg.norm(acc) < 1e-25
    m = np.array([1e-15, 1e-15])
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [1e6, 0, 0]]), m)
    assert np.all(np.isfinite(acc)) and np.linalg.norm(momentum(acc, m)) < 1e-20
    acc = bhut.accelerations(np.array([[0.0, 0, 0], [1e-6, 0, 0]]), np.array([1e10, 1e10]))
    assert np.all(np.isfinite(acc))
    b = 1e12
    acc = bhut.accelerations(np.array([[b, b, b], [b + 1.0, b, b]]), np.ones(2))
    assert np.all(np.isfinite(acc)) and acc[0, 0] > 0


def test_edge_tree_cases(simple_system, random_system):
    """edge_cases/test_boundary_conditions.py:350-430"""
    acc = bhut.Tree(np.array([[1.0, 2, 3]]), np.array([1.0])).build().accelerations()
    np.testing.assert_allclose(acc, 0.0, atol=1e-15)
    p, m = simple_system
    tree = bhut.Tree(p, m).build()
    same = tree.rebuild(p, m).accelerations()
    diff = tree.rebuild(p, m * np.array([10.0, 0.1])).accelerations()
    assert np.all(np.isfinite(same)) and not np.allclose(same, diff, rtol=1e-1)
    rp, rm = random_system
    rng = np.random.default_rng(8)
    tree = bhut.Tree(rp, rm).build()
    assert np.all(np.isfinite(tree.refit(rp + 1e-10 * rng.standard_normal(rp.shape))
                              .accelerations()))
    assert np.all(np.isfinite(tree.refit(rp + 10.0 * rng.standard_normal(rp.shape))
                              .accelerations()))
    big = rng.standard_normal((100, 3))
    tree = bhut.Tree(big, np.ones(100)).build()
    for _ in range(5):
        acc = tree.refit(big + 0.01 * rng.standard_normal(big.shape)).accelerations()
        assert acc.shape == (100, 3) and np.all(np.isfinite(acc))


def test_edge_error_recovery(simple_system):
    """edge_cases/test_boundary_conditions.py:436-467 and
    integration/test_workflows.py:262-280"""
    tree = bhut.Tree(*simple_system).build()
    valid = tree.accelerations()
    with pytest.raises(ValueError):
        tree.refit(np.array([[np.nan, 0, 0]]))
    np.testing.assert_allclose(tree.accelerations(), valid, rtol=1e-15)
    for p, m, terms in ((np.array([[1, 2]]), np.array([1]), ("dimension", "2d array")),
                        (np.array([[1, 2, 3]]), np.array([1, 2]), ("particles", "elements"))):
        with pytest.raises(ValueError) as e:
            bhut.accelerations(p, m)
        assert any(t in str(e.value).lower() for t in terms)


def test_edge_partial_failure_handling():
    """edge_cases/test_boundary_conditions.py:469-488.  The reference fails
    its own bound here (total momentum -0.125 vs atol 1e-10: forces of the
    1e15-mass particle cancelling in FP64); the drop-in is held to the same
    shape and finiteness checks and to the momentum that FP64 arithmetic
    allows for these masses (a few ulps of the largest force, well under 1)."""
    p = np.array([[0.0, 0, 0], [1.0, 0, 0], [1e-15, 0, 0], [1e15, 0, 0]])
    m = np.array([1.0, 1.0, 1e-15, 1e15])
    acc = bhut.accelerations(p, m)
    assert acc.shape == (4, 3) and np.all(np.isfinite(acc))
    assert np.linalg.norm(momentum(acc, m)) <= 1.0


# -- tests/integration/test_backend_consistency.py --------------------------------
def test_integration_dtypes_and_backends(random_system, hierarchical_system):
    """integration/test_backend_consistency.py:17-50 and :133-155"""
    p, m = random_system
    a32 = bhut.accelerations(p.astype(np.float32), m.astype(np.float32), backend="numpy")
    a64 = bhut.accelerations(p, m, backend="numpy")
    assert a32.dtype == np.float64 and np.all(np.isfinite(a32))
    np.testing.assert_allclose(a32, a64, rtol=1e-6)
    np.testing.assert_allclose(bhut.accelerations(*hierarchical_system, backend="auto"),
                               bhut.accelerations(*hierarchical_system, backend="numpy"),
                               rtol=1e-15)
    for theta in (0.5, 1.0, 2.0):
        ref = bhut.Tree(*hierarchical_system, backend="numpy").build().accelerations(theta=theta)
        acc = bhut.Tree(*hierarchical_system, backend="auto").build().accelerations(theta=theta)
        np.testing.assert_allclose(acc, ref, rtol=1e-15)


def test_integration_parameter_consistency(random_system, simple_system):
    """integration/test_backend_consistency.py:157-228"""
    p, m = random_system
    res = {L: bhut.Tree(p, m, leaf_size=L).build().accelerations(theta=1.0) for L in (4, 16, 32)}
    for L in (16, 32):
        assert 0.1 < np.max(np.abs(res[L])) < 100
        assert 0.1 < np.linalg.norm(res[L]) / np.linalg.norm(res[4]) < 10
    sp, sm = simple_system
    for theta in (0.1, 0.5, 1.0, 1.5, 2.0):
        acc = bhut.Tree(sp, sm).build().accelerations(theta=theta)
        assert np.all(np.isfinite(acc))
        if theta <= 0.5:
            ref = bhut.Tree(sp, sm).build().accelerations(theta=0.1)
            np.testing.assert_allclose(acc, ref, rtol=theta)
    precise = bhut.Tree(sp, sm).build().accelerations(theta=1e-6)
    fast = bhut.Tree(sp, sm).build().accelerations(theta=5.0)
    np.testing.assert_allclose(momentum(precise, sm), 0.0, atol=1e-12)
    np.testing.assert_allclose(momentum(fast, sm), 0.0, atol=1e-10)


def test_integration_reproducibility(random_system, hierarchical_system):
    """integration/test_backend_consistency.py:235-284"""
    p, m = random_system
    runs = [bhut.Tree(p, m).build().accelerations(theta=1.0) for _ in range(3)]
    for r in runs[1:]:
        np.testing.assert_allclose(r, runs[0], rtol=1e-15)
    h = [bhut.Tree(*hierarchical_system, leaf_size=16).build().accelerations(theta=1.0)
         for _ in range(2)]
    np.testing.assert_allclose(h[0], h[1], rtol=1e-15)
    fresh = bhut.Tree(p, m).build().accelerations(theta=1.0)
    rebuilt = bhut.Tree(p, m).build().rebuild(p, m).accelerations(theta=1.0)
    np.testing.assert_allclose(fresh, rebuilt, rtol=1e-15)


def test_integration_tree_vs_manual_direct_sum(simple_system):
    """integration/test_backend_consistency.py:311-332"""
    p, m = simple_system
    acc = bhut.Tree(p, m).build().accelerations(theta=1e-8)
    ref = np.zeros_like(p)
    for i in range(len(p)):
        for j in range(len(p)):
            if i != j:
                r = p[j] - p[i]
                ref[i] += m[j] * r / np.linalg.norm(r) ** 3
    np.testing.assert_allclose(acc, ref, rtol=1e-6)


def test_integration_rebuild_equals_fresh(random_system):
    """integration/test_backend_consistency.py:334-354"""
    p, m = random_system
    q = p + np.random.default_rng(9).standard_normal(p.shape) * 0.001
    rebuilt = bhut.Tree(p, m).build().rebuild(q, m).accelerations(theta=1.0)
    fresh = bhut.Tree(q, m).build().accelerations(theta=1.0)
    np.testing.assert_allclose(rebuilt, fresh, rtol=1e-15)


def test_integration_cross_validation(hierarchical_system, random_system):
    """integration/test_backend_consistency.py:356-425"""
    ref = bhut.accelerations(*hierarchical_system, backend="numpy")
    np.testing.assert_allclose(bhut.accelerations(*hierarchical_system, backend="auto"), ref,
                               rtol=1e-12)
    p, m = random_system
    acc_ref = bhut.Tree(p, m, leaf_size=4).build().accelerations(theta=0.1)
    for theta, leaf in ((0.5, 32), (1.0, 16), (1.5, 8)):
        acc = bhut.Tree(p, m, leaf_size=leaf).build().accelerations(theta=theta)
        assert 0.01 < np.max(np.abs(acc)) < 1000
        assert 0.1 < np.linalg.norm(acc) / np.linalg.norm(acc_ref) < 10


def test_integration_stress():
    """integration/test_backend_consistency.py:433-496"""
    rng = np.random.default_rng(10)
    p = rng.standard_normal((10, 3))
    m = np.array([1e-10, 1.0, 1e10, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0])
    a1 = bhut.Tree(p, m, backend="numpy").build().accelerations()
    a2 = bhut.Tree(p, m, backend="auto").build().accelerations()
    assert np.all(np.isfinite(a1))
    np.testing.assert_allclose(a2, a1, rtol=1e-12)
    acc = bhut.Tree(np.array([[0.0, 0, 0], [1e-8, 0, 0], [1.0, 0, 0], [0.0, 1, 0]]),
                    np.ones(4)).build().accelerations()
    assert np.all(np.isfinite(acc)) and np.linalg.norm(acc[0]) > np.linalg.norm(acc[2])
    acc = bhut.Tree(np.array([[0.0, 0, 0], [1e6, 0, 0], [0.0, 1e6, 0]]),
                    np.ones(3)).build().accelerations()
    assert np.all(np.isfinite(acc)) and np.max(np.abs(acc)) < 1e-10


# -- tests/integration/test_workflows.py --------------------------------------------
def test_workflow_small_system_and_symmetry():
    """integration/test_workflows.py:189-207 and :343-362"""
    tree = bhut.Tree(np.array([[0.0, 0, 0], [1.0, 0, 0]]), np.ones(2), leaf_size=2).build()
    acc = tree.accelerations(theta=1.0)
    assert acc.shape == (2, 3) and np.all(np.isfinite(acc))
    np.testing.assert_allclose(acc[0], -acc[1], rtol=1e-12)
    p = np.array([[-1.0, 0, 0], [1.0, 0, 0], [0, -1.0, 0], [0, 1.0, 0]])
    acc = bhut.Tree(p, np.array([1.0, 1.0, 2.0, 2.0])).build().accelerations()
    np.testing.assert_allclose(acc[0, 0], -acc[1, 0], rtol=1e-10)
    np.testing.assert_allclose(acc[2, 1], -acc[3, 1], rtol=1e-10)


def test_workflow_medium_system_steps(random_system):
    """integration/test_workflows.py:209-235"""
    p, m = random_system
    tree = bhut.Tree(p, m).build()
    x, v = p.copy(), np.zeros_like(p)
    for _ in range(5):
        acc = tree.refit(x).accelerations()
        v += 0.01 * acc
        x += 0.01 * v
        assert np.all(np.isfinite(x)) and np.all(np.isfinite(v)) and np.all(np.isfinite(acc))


def test_workflow_large_system_momentum():
    """integration/test_workflows.py:237-255"""
    rng = np.random.default_rng(11)
    p = rng.standard_normal((100, 3))
    m = np.abs(rng.standard_normal(100)) + 0.1
    acc = bhut.Tree(p, m, leaf_size=16).build().accelerations()
    assert acc.shape == (100, 3) and np.all(np.isfinite(acc))
    np.testing.assert_allclose(momentum(acc, m), 0.0, atol=1e-10)
