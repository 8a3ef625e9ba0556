"""compute_tree_statistics (bhut/traverse/bh.py:604-700) on the GPU against
the reference's own values (golden fixture) and the oracle."""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import workloads
from test_oracle_golden import stats_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


def test_statistics_match_reference(golden_stats):
    n = 0
    for tag, pos, m, L, theta, want in stats_cases(golden_stats):
        td = bh.build_tree(pos, m, leaf_size=L, backend="auto", dim=pos.shape[1])
        st = bh.compute_tree_statistics(td, pos, theta)
        got = np.array([st["avg_nodes_visited"], st["avg_particles_computed"],
                        st["avg_monopoles_used"], st["total_operations"]])
        assert np.array_equal(got, want), (tag, got, want)
        n += 1
    assert n == 24


def test_statistics_large_against_oracle(oracle_mod):
    pos, m = workloads.plummer(200_000, seed=9)
    tree = bh.Tree(pos, m, leaf_size=32).build()
    tg = workloads.cube_targets(20_000, seed=3, side=6.0)
    for theta in (0.3, 0.7):
        st = bh.compute_tree_statistics(tree, tg, theta)
        nodes, parts, monos = oracle_mod.tree_statistics(tree._tree, tg, theta)
        assert st["total_operations"] == parts + monos
        assert st["avg_nodes_visited"] == nodes / len(tg)
        assert st["avg_monopoles_used"] == monos / len(tg)
    with pytest.raises(ZeroDivisionError):
        bh.compute_tree_statistics(tree, np.zeros((0, 3)), 0.5)
    tree.close()


@pytest.mark.parametrize("form", ["exact", "fast", "fp32"])
def test_target_chunks_in_chunks_out(form):
    pos, m = workloads.gaussian(30_000, seed=4)
    tg = workloads.cube_targets(10_000, seed=5, side=8.0)
    tree = bh.Tree(pos, m, form=form).build()
    whole = tree.accelerations(tg, theta=0.6, softening=0.01)
    sizes = [1, 4095, 33, 5000, 871]
    chunks = np.split(tg, np.cumsum(sizes)[:-1])
    got = tree.accelerations_chunks(chunks, theta=0.6, softening=0.01)
    assert [len(c) for c in got] == sizes
    assert np.array_equal(np.concatenate(got), whole)
    tree.close()


def test_self_chunks_match_targets_path():
    pos, m = workloads.plummer(20_000, seed=6)
    sizes = [7000, 6000, 7000]
    pc = np.split(pos, np.cumsum(sizes)[:-1])
    mc = np.split(m, np.cumsum(sizes)[:-1])
    got = bh.accelerations_chunks(pc, mc, theta=0.5, softening=0.01, form="exact")
    whole = bh.accelerations(pos, m, theta=0.5, softening=0.01, form="exact")
    assert [len(c) for c in got] == sizes
    # evaluated as external targets: same interactions, own pair adds zero
    from conftest import rel_l2
    assert rel_l2(np.concatenate(got), whole) < 1e-14
