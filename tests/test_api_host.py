"""Host-side validation of the public API (no GPU needed: every case raises
before the engine is called).  Messages follow bhut/api.py:84-152,254-364,
432-786 and tests/edge_cases/test_boundary_conditions.py of the reference."""
import numpy as np
import pytest

import bhut_gb300 as bh

POS = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 1.0, 0]])
M = np.ones(3)


@pytest.mark.parametrize("kw,msg", [
    ({"criterion": "xx"}, "criterion must be 'bh'"),
    ({"multipole": "quad"}, "multipole must be 'mono'"),
    ({"backend": "cupy"}, "Unsupported backend"),
    ({"dim": 4}, "dim must be 2 or 3"),
    ({"softening": -1.0}, "softening must be non-negative"),
    ({"theta": -0.5}, "theta must be non-negative"),
    ({"leaf_size": 0}, "leaf_size must be positive"),
    ({"softening": np.array([0.1, 0.2, 0.3])}, "Variable softening per particle"),
    ({"softening": np.array([0.1, 0.2])}, "softening array has 2 elements but need 3"),
    ({"dim": 2}, "positions has 3 dimensions but dim=2"),
])
def test_accelerations_argument_errors(kw, msg):
    with pytest.raises(ValueError, match=msg):
        bh.accelerations(POS, M, **kw)


def test_shape_errors():
    with pytest.raises(ValueError, match="positions must be 2D array"):
        bh.accelerations(np.zeros(3), np.ones(3))
    with pytest.raises(ValueError, match="masses must be 1D array"):
        bh.accelerations(POS, np.ones((3, 1)))
    with pytest.raises(ValueError, match="positions has 3 particles but masses has 2 elements"):
        bh.accelerations(POS, np.ones(2))


def test_empty_input():
    with pytest.raises(ValueError, match="empty|zero"):
        bh.accelerations(np.zeros((0, 3)), np.zeros(0))


def test_non_numeric_parameters():
    with pytest.raises((TypeError, ValueError)):
        bh.accelerations(POS, M, theta="0.5")
    with pytest.raises((TypeError, ValueError)):
        bh.accelerations(POS, M, leaf_size="32")


def test_tree_lifecycle_errors():
    t = bh.Tree(POS, M)
    assert t._tree is None and not t._is_built
    assert t.dim == 3 and t.leaf_size == 32 and t.backend == "auto"
    with pytest.raises(ValueError, match="Tree must be built before evaluating accelerations"):
        t.accelerations()
    with pytest.raises(ValueError, match="Tree must be built before refitting"):
        t.refit(POS)
    with pytest.raises(RuntimeError, match="Tree not built"):
        t.evaluate_accelerations(0.0)
    with pytest.raises(ValueError, match="dim must be 2 or 3"):
        bh.Tree(POS, M, dim=1)
    with pytest.raises(ValueError, match="leaf_size must be positive"):
        bh.Tree(POS, M, leaf_size=-1)
    with pytest.raises(ValueError, match="Unsupported backend"):
        bh.Tree(POS, M, backend="jax")


def test_inputs_converted_to_float64():
    t = bh.Tree(POS.astype(np.float32), np.ones(3, dtype=np.int64))
    assert t.positions.dtype == np.float64 and t.masses.dtype == np.float64


def test_form_names():
    with pytest.raises(ValueError, match="form must be one of"):
        bh.Tree(POS, M, form="fp16")
