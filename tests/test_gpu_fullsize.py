"""The batched and precision forms at the sizes of their named workloads.

* Batched: 2,048 Plummer spheres, N log-uniform in [256, 65,536] (about 22.6M
  particles, 64-bit offsets, 2,048 sort segments, the persistent task queue
  at full length), one CUDA-graph solve of the FP32 form with quadrupoles.
  A seeded sample of 32 systems -- the largest and the smallest among them --
  must equal single-system solves bit for bit; the float-float form of the
  same batch is checked against the oracle (the C restatement of
  bhut/traverse/bh.py) on 8 systems to 1e-11 relative L2.
* Precision: the 4M-particle galaxy (70 % exponential disc, 30 % Hernquist
  bulge), softening 0.005, theta 0.5: the FP32 form against the
  FP64-accurate form on all targets (median relative error <= 1e-7), and the
  FP64-accurate form against the oracle on 4,096 sampled targets (relative
  L2 <= 1e-10).
"""
import numpy as np
import pytest

import bhut_gb300 as bh
from bhut_gb300 import batch, workloads
from conftest import rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


@pytest.fixture(scope="module")
def c4_systems():
    return workloads.plummer_batch(2048, 256, 65536, seed=11)


def test_batched_2048_systems_equal_single_solves(c4_systems):
    import torch
    pos, m, off = batch.concat_systems(c4_systems)
    assert off[-1] > 2**24                 # tens of millions of particles
    pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
    sv = batch.BatchedSolver(leaf_size=16, form="fp32", multipole="quad", use_graph=True,
                             targets_per_warp=32, stack="shared")
    sv.load(pd, md, off)
    acc = sv.solve(theta=0.5, softening=0.01)
    acc2 = sv.solve(theta=0.5, softening=0.01)       # graph replay
    assert torch.equal(acc, acc2)
    acc = acc.cpu().numpy()
    sv.close()
    sizes = np.diff(off)
    rng = np.random.default_rng(4)
    pick = set(rng.choice(len(c4_systems), 30, replace=False).tolist())
    pick |= {int(np.argmax(sizes)), int(np.argmin(sizes))}
    for s in sorted(pick):
        p, mm = c4_systems[s]
        ref = bh.accelerations(p, mm, theta=0.5, softening=0.01, form="fp32",
                               multipole="quad", leaf_size=16)
        assert np.array_equal(acc[off[s]:off[s + 1]], ref), (s, sizes[s])


def test_batched_2048_systems_fast_form_vs_oracle(c4_systems, oracle_mod):
    import torch
    pos, m, off = batch.concat_systems(c4_systems)
    sv = batch.BatchedSolver(leaf_size=32, form="fast", use_graph=True)
    sv.load(torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda(), off)
    acc = sv.solve(theta=0.5, softening=0.01).cpu().numpy()
    sv.close()
    sizes = np.diff(off)
    # eight systems across the lower 60 % of the size range (the oracle
    # traverses every target of each)
    order = np.argsort(sizes)
    pick = order[np.linspace(0, len(order) * 0.6, 8).astype(int)]
    for s in pick:
        p, mm = c4_systems[s]
        tree = oracle_mod.build_tree(p, mm, 32)
        ref = oracle_mod.accelerations(tree, p, mm, theta=0.5, softening=0.01)
        assert rel_l2(acc[off[s]:off[s + 1]], ref) <= 1e-11, (s, sizes[s])


@pytest.fixture(scope="module")
def galaxy4m():
    return workloads.galaxy(4_000_000, seed=7)


def test_galaxy_4m_fp32_vs_fast_and_fast_vs_oracle(galaxy4m, oracle_mod):
    import torch
    from bhut_gb300 import precision
    pos, m = galaxy4m
    pd, md = torch.as_tensor(pos).cuda(), torch.as_tensor(m).cuda()
    t32 = bh.Tree(pd, md, leaf_size=16, form="fp32").build()
    a32 = t32.accelerations(theta=0.5, softening=0.005).cpu().numpy()
    t32.close()
    t64 = bh.Tree(pd, md, leaf_size=16, form="fast").build()
    a64 = t64.accelerations(theta=0.5, softening=0.005).cpu().numpy()
    t64.close()
    dist = precision.error_distribution(a32, a64)
    assert dist["median"] <= 1e-7, dist
    idx = precision.sample_indices(len(m), 4096, seed=3)
    tree = oracle_mod.build_tree(pos, m, 16)
    ref = oracle_mod.accelerations(tree, pos, m, theta=0.5, softening=0.005, self_index=idx)
    assert rel_l2(a64[idx], ref) <= 1e-10
