"""The CPU oracle against the reference's own outputs (golden fixtures).

Pins oracle/bhut_oracle.c: Morton keys, permutation and every TreeData array
bit-exact; accelerations to 1e-12 relative (the fixtures come from the
reference's pure-NumPy pair kernel, the oracle follows the Numba loop, so the
two differ only in the last bits of each term).
"""
import hashlib

import numpy as np
import pytest

from conftest import TREE_FIELDS, rel_l2

FORCE_RTOL = 1e-12


def _tree_equal(o, g, prefix):
    for f in TREE_FIELDS:
        a = np.asarray(getattr(o, f))
        b = g[prefix + f]
        assert a.shape == b.shape, (prefix, f, a.shape, b.shape)
        assert np.array_equal(a.astype(b.dtype), b), f"{prefix}{f} differs"


def test_small_systems_tree_and_forces(oracle_mod, golden_small):
    g = golden_small
    checked = 0
    for name in g["names"]:
        pos, m = g[f"{name}__pos"], g[f"{name}__masses"]
        assert np.array_equal(oracle_mod.morton_codes(pos), g[f"{name}__keys"]), name
        tg = g[f"{name}__targets"]
        for L in (1, 4, 32):
            t = oracle_mod.build_tree(pos, m, L)
            _tree_equal(t, g, f"{name}__L{L}__")
            for theta in (0.0, 0.7):
                for eps in (0.0, 0.01):
                    tag = f"{name}__L{L}__t{theta}__e{eps}"
                    got = oracle_mod.accelerations(t, pos, m, theta=theta, softening=eps)
                    assert rel_l2(got, g[tag + "__self"]) <= FORCE_RTOL, tag
                    got = oracle_mod.accelerations(t, pos, m, theta=theta, softening=eps,
                                                   targets=tg)
                    assert rel_l2(got, g[tag + "__ext"]) <= FORCE_RTOL, tag
                    checked += 1
    assert checked >= 80


def test_gauss10k(oracle_mod, golden_gauss):
    g = golden_gauss
    pos, m = g["pos"], g["masses"]
    L, eps = int(g["leaf_size"]), float(g["softening"])
    assert np.array_equal(oracle_mod.morton_codes(pos), g["keys"])
    t = oracle_mod.build_tree(pos, m, L)
    _tree_equal(t, g, "tree_")
    got = oracle_mod.accelerations(t, pos, m, theta=0.5, softening=eps, self_index=g["sample"])
    assert rel_l2(got, g["acc_theta05"]) <= FORCE_RTOL
    got = oracle_mod.accelerations(t, pos, m, theta=0.0, softening=eps, self_index=g["sample0"])
    assert rel_l2(got, g["acc_theta0"]) <= FORCE_RTOL
    got = oracle_mod.accelerations(t, pos, m, theta=0.5, softening=eps, targets=g["targets"])
    assert rel_l2(got, g["acc_targets_theta05"]) <= FORCE_RTOL
    # theta = 0 is direct summation (bh.py:599-601: every node opens)
    direct = oracle_mod.direct_sum(pos, m, softening=eps, self_index=g["sample0"])
    assert rel_l2(direct, g["acc_theta0"]) <= 1e-13


def test_refit_cases(oracle_mod, golden_refit):
    g = golden_refit
    for tag in ("plain", "negmass"):
        pos, m = g[f"{tag}__pos"], g[f"{tag}__masses"]
        pos2, m2 = g[f"{tag}__pos2"], g[f"{tag}__masses2"]
        t = oracle_mod.build_tree(pos, m, 16)
        assert oracle_mod.should_refit(t, pos2)
        r = oracle_mod.refit(t, pos2, m2)
        _tree_equal(r, g, f"{tag}__refit__")
        got = oracle_mod.accelerations(r, pos2, m2, theta=0.5, softening=0.01,
                                       self_index=g[f"{tag}__sample"])
        assert rel_l2(got, g[f"{tag}__acc"]) <= FORCE_RTOL
    # a large move makes refit fall back to a rebuild (refit.py:236-249)
    pos, m, pos3 = g["moved__pos"], g["moved__masses"], g["moved__pos3"]
    t = oracle_mod.build_tree(pos, m, 8)
    assert not oracle_mod.should_refit(t, pos3)
    _tree_equal(oracle_mod.build_tree(pos3, m, 8), g, "moved__tree__")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.slow
def test_plummer_1m_digests(oracle_mod, golden_plummer):
    """N=1,000,000 Plummer: keys, perm and tree arrays match the reference's
    by SHA-256; 12 sampled accelerations to 1e-12."""
    from bhut_gb300 import workloads
    g = golden_plummer
    dig = dict(zip(g["digest_names"], g["digest_values"]))
    pos, m = workloads.plummer(int(g["n"]), seed=int(g["seed"]))
    assert _digest(pos) == dig["pos"], "Plummer generator drifted"
    t = oracle_mod.build_tree(pos, m, int(g["leaf_size"]))
    assert len(t.mass) == int(g["num_nodes"])
    assert _digest(oracle_mod.morton_codes(pos)) == dig["keys"]
    for f in TREE_FIELDS:
        a = np.asarray(getattr(t, f))
        a = a.astype(np.int64) if a.dtype.kind == "i" else a
        assert _digest(a) == dig[f], f
    got = oracle_mod.accelerations(t, pos, m, theta=0.5, softening=float(g["softening"]),
                                   self_index=g["sample"])
    assert rel_l2(got, g["acc_theta05"]) <= FORCE_RTOL


def test_known_answers(oracle_mod):
    """Known answers of tests/validation/test_physics_validation.py:17-48 and
    :414-432 of the reference, evaluated by the oracle."""
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    m = np.ones(2)
    t = oracle_mod.build_tree(pos, m, 32)
    a = oracle_mod.accelerations(t, pos, m, theta=0.5, softening=0.0)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, rtol=1e-10)
    pos = np.array([[0.0, 0, 0], [1e6, 0, 0]])
    t = oracle_mod.build_tree(pos, m, 32)
    a = oracle_mod.accelerations(t, pos, m, theta=0.5, softening=0.0)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1e-12, rtol=1e-10)


def stats_cases(g):
    """(tag, positions, masses, leaf_size, theta, reference values) of the
    compute_tree_statistics fixture."""
    for tag in g["names"]:
        name, L, t = str(tag).split("__")
        yield (str(tag), g[f"{name}__pos"], g[f"{name}__masses"], int(L[1:]), float(t[1:]),
               g[str(tag)])


def test_tree_statistics(oracle_mod, golden_stats):
    n_cases = 0
    for tag, pos, m, L, theta, want in stats_cases(golden_stats):
        t = oracle_mod.build_tree(pos, m, L)
        nodes, parts, monos = oracle_mod.tree_statistics(t, pos, theta)
        n = len(pos)
        got = np.array([nodes / n, parts / n, monos / n, parts + monos])
        assert np.array_equal(got, want), (tag, got, want)
        n_cases += 1
    assert n_cases == 24
