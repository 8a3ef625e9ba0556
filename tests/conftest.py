"""Test configuration: markers, paths and shared fixtures."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA engine")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def engine_lib():
    """Builds (if stale) and loads libbhut_gb300.so."""
    from bhut_gb300 import _build, _lib
    _build.build()
    return _lib.load()


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


@pytest.fixture(scope="session")
def golden_small():
    return load_golden("small_systems")


@pytest.fixture(scope="session")
def golden_gauss():
    return load_golden("gauss10k_L32")


@pytest.fixture(scope="session")
def golden_refit():
    return load_golden("refit_cases")


@pytest.fixture(scope="session")
def golden_plummer():
    return load_golden("plummer1m_digest")


@pytest.fixture(scope="session")
def golden_stats():
    return load_golden("tree_statistics")


TREE_FIELDS = ["center", "half_size", "mass", "com", "first_child", "child_count", "start",
               "count", "is_leaf", "perm"]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    if den == 0.0:
        return 0.0 if num == 0.0 else np.inf
    return num / den
