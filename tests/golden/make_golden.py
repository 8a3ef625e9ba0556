"""Generate the golden fixtures in this folder by running the reference itself.

Usage (needs the bhut 0.1.0 source tree; it is imported read-only):

    BHUT_REFERENCE=<path of the bhut source tree> python tests/golden/make_golden.py

Every fixture stores the inputs (or the seed plus a digest of the inputs for
the 1,000,000-particle case), the reference's Morton keys, permutation and
TreeData arrays, and reference accelerations on sampled targets computed with
``bhut.traverse.bh._barnes_hut_single_target`` /
``_barnes_hut_single_target_external`` (the per-target loops of
bhut/traverse/bh.py:485-548 and :83-146).  The reference runs its pure-NumPy
leaf loop here (Numba is not installed), which differs from the Numba loop
only in the last bits of each pair term.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if not os.environ.get("BHUT_REFERENCE"):
    sys.exit("set BHUT_REFERENCE to the bhut 0.1.0 source tree (the folder holding bhut/)")
sys.path.insert(0, os.environ["BHUT_REFERENCE"])
sys.path.insert(0, REPO)

import bhut  # noqa: E402
from bhut.backends.numpy_ import numpy_namespace  # noqa: E402
from bhut.space.bbox import aabb, normalize_to_unit  # noqa: E402
from bhut.traverse import bh  # noqa: E402
from bhut.tree.build import build_tree  # noqa: E402
from bhut.utils.morton import morton_codes  # noqa: E402

from bhut_gb300 import workloads  # noqa: E402

TREE_FIELDS = ["center", "half_size", "mass", "com", "first_child", "child_count", "start",
               "count", "is_leaf", "perm"]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_tree(pos, m, L):
    return build_tree(pos, m, dim=pos.shape[1], leaf_size=L, xp=numpy_namespace)


def tree_dict(t, prefix="tree_"):
    out = {}
    for f in TREE_FIELDS:
        a = np.asarray(getattr(t, f))
        out[prefix + f] = a.astype(np.int64) if a.dtype.kind == "i" else a
    return out


def ref_self(t, pos, m, idx, theta, eps, G=1.0):
    return np.array([bh._barnes_hut_single_target(t, pos[i], int(i), pos, m, eps, theta, G)
                     for i in idx]).reshape(len(idx), pos.shape[1])


def ref_ext(t, pos, m, tg, theta, eps, G=1.0):
    return np.array([bh._barnes_hut_single_target_external(t, pos, m, x, eps, theta, G)
                     for x in tg]).reshape(len(tg), pos.shape[1])


def keys_of(pos):
    pmin, pmax = aabb(pos)
    return morton_codes(normalize_to_unit(pos, pmin, pmax))


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}.npz ({os.path.getsize(path) / 1024:.0f} KiB)")


def case_gauss10k():
    """N=10,000 standard normal (seed 0), unit masses, L=32, eps=0.01."""
    pos, m = workloads.gaussian(10_000, seed=0)
    L, eps = 32, 0.01
    t = ref_tree(pos, m, L)
    rng = np.random.default_rng(100)
    idx = np.sort(rng.choice(len(pos), 256, replace=False))
    idx0 = idx[:48]
    tg = workloads.cube_targets(64, seed=101, side=8.0)
    save("gauss10k_L32", pos=pos, masses=m, leaf_size=L, softening=eps, keys=keys_of(pos),
         sample=idx, acc_theta05=ref_self(t, pos, m, idx, 0.5, eps),
         sample0=idx0, acc_theta0=ref_self(t, pos, m, idx0, 0.0, eps),
         targets=tg, acc_targets_theta05=ref_ext(t, pos, m, tg, 0.5, eps),
         **tree_dict(t))


def small_systems():
    rng = np.random.default_rng(7)
    cases = {}
    for n in (1, 2, 3, 7, 31, 32, 33, 65, 100, 257):
        cases[f"normal_n{n}"] = (rng.standard_normal((n, 3)), rng.uniform(0.5, 2.0, n))
    planar = rng.standard_normal((40, 3))
    planar[:, 2] = 0.0
    cases["planar_n40"] = (planar, np.ones(40))
    dup = rng.standard_normal((20, 3))
    dup[10:] = dup[:10]
    cases["duplicates_n20"] = (dup, np.ones(20))
    zm = rng.standard_normal((50, 3))
    mz = np.ones(50)
    mz[::3] = 0.0
    cases["zero_masses_n50"] = (zm, mz)
    cases["all_zero_mass_n9"] = (rng.standard_normal((9, 3)), np.zeros(9))
    cases["mass_range_n16"] = (rng.standard_normal((16, 3)), np.logspace(-15, 15, 16))
    cases["clustered_n6"] = (5.0 + 1e-8 * rng.standard_normal((6, 3)), np.ones(6))
    cases["far_pair"] = (np.array([[0.0, 0, 0], [1e15, 0, 0]]), np.array([1.0, 1.0]))
    cases["normal2d_n300"] = (rng.standard_normal((300, 2)), rng.uniform(0.5, 2.0, 300))
    cases["line2d_n33"] = (np.stack([np.linspace(-1, 1, 33), np.zeros(33)], 1), np.ones(33))
    return cases


def case_small():
    """Small systems: full trees and all self accelerations for several
    (leaf_size, theta, softening) settings, plus external targets."""
    out = {}
    names = []
    for name, (pos, m) in small_systems().items():
        names.append(name)
        dim = pos.shape[1]
        out[f"{name}__pos"] = pos
        out[f"{name}__masses"] = m
        out[f"{name}__keys"] = keys_of(pos)
        tg = np.random.default_rng(len(name)).standard_normal((12, dim)) * 1.5
        out[f"{name}__targets"] = tg
        for L in (1, 4, 32):
            t = ref_tree(pos, m, L)
            for k, v in tree_dict(t, prefix="").items():
                out[f"{name}__L{L}__{k}"] = v
            for theta in (0.0, 0.7):
                for eps in (0.0, 0.01):
                    tag = f"{name}__L{L}__t{theta}__e{eps}"
                    out[tag + "__self"] = ref_self(t, pos, m, np.arange(len(pos)), theta, eps,
                                                   G=1.0)
                    out[tag + "__ext"] = ref_ext(t, pos, m, tg, theta, eps, G=1.0)
    out["names"] = np.array(names)
    save("small_systems", **out)


def case_refit():
    """Tree.refit after a small move (refit path) and after a large move
    (refit falls back to rebuild, refit.py:236-249); negative masses exercise
    the refit rule that skips children with non-positive mass."""
    rng = np.random.default_rng(11)
    out = {}
    for tag, n, neg in (("plain", 3000, False), ("negmass", 500, True)):
        pos = rng.standard_normal((n, 3))
        m = rng.uniform(0.5, 1.5, n)
        if neg:
            m[::7] *= -1.0
        pos2 = pos + 0.01 * rng.standard_normal((n, 3))
        m2 = m * rng.uniform(0.9, 1.1, n)
        tr = bhut.Tree(pos, m, leaf_size=16)
        tr.build()
        tr.refit(pos2, m2)
        t = tr._tree
        idx = np.arange(0, n, max(1, n // 64))
        out.update({f"{tag}__pos": pos, f"{tag}__masses": m, f"{tag}__pos2": pos2,
                    f"{tag}__masses2": m2, f"{tag}__sample": idx,
                    f"{tag}__acc": ref_self(t, pos2, m2, idx, 0.5, 0.01)})
        for k, v in tree_dict(t, prefix="").items():
            out[f"{tag}__refit__{k}"] = v
    # large move: refit -> rebuild
    pos = rng.standard_normal((400, 3))
    m = np.ones(400)
    tr = bhut.Tree(pos, m, leaf_size=8)
    tr.build()
    pos3 = pos * 3.0
    tr.refit(pos3)
    out.update({"moved__pos": pos, "moved__masses": m, "moved__pos3": pos3})
    for k, v in tree_dict(tr._tree, prefix="").items():
        out[f"moved__tree__{k}"] = v
    save("refit_cases", **out)


def case_plummer_1m():
    """N=1,000,000 Plummer (seed 1): digests of keys, perm and the tree
    arrays, plus 12 sampled self accelerations at theta=0.5, eps=0.01."""
    n, L, eps = 1_000_000, 32, 0.01
    pos, m = workloads.plummer(n, seed=1)
    t0 = time.time()
    t = ref_tree(pos, m, L)
    print(f"reference build at N=1M: {time.time() - t0:.2f} s")
    keys = keys_of(pos)
    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(n, 12, replace=False))
    t0 = time.time()
    acc = ref_self(t, pos, m, idx, 0.5, eps)
    print(f"reference traversal: {(time.time() - t0) / len(idx):.3f} s/target")
    digests = {"pos": digest(pos), "masses": digest(m), "keys": digest(keys)}
    for f in TREE_FIELDS:
        a = np.asarray(getattr(t, f))
        digests[f] = digest(a.astype(np.int64) if a.dtype.kind == "i" else a)
    save("plummer1m_digest", seed=1, n=n, leaf_size=L, softening=eps, sample=idx,
         acc_theta05=acc, sample_pos=pos[idx], num_nodes=len(t.mass),
         digest_names=np.array(list(digests.keys())),
         digest_values=np.array(list(digests.values())))


def case_statistics():
    """compute_tree_statistics (bh.py:604-700) of the reference on its own
    trees: a 3,000-particle Gaussian (L=32 and L=8, theta 0.5 and 0.9), a
    2-D case, and small systems with zero masses and duplicates."""
    from bhut.traverse.bh import compute_tree_statistics
    out = {}
    rng = np.random.default_rng(23)
    cases = {"gauss3k": (rng.standard_normal((3000, 3)), np.ones(3000)),
             "gauss2d_1k": (rng.standard_normal((1000, 2)), rng.uniform(0.5, 2.0, 1000))}
    small = small_systems()
    for k in ("zero_masses_n50", "duplicates_n20", "normal_n1", "all_zero_mass_n9"):
        cases[k] = small[k]
    names = []
    for name, (pos, m) in cases.items():
        out[f"{name}__pos"] = pos
        out[f"{name}__masses"] = m
        for L in (32, 8):
            t = ref_tree(pos, m, L)
            for theta in (0.5, 0.9):
                st = compute_tree_statistics(t, pos, theta)
                tag = f"{name}__L{L}__t{theta}"
                names.append(tag)
                out[tag] = np.array([st["avg_nodes_visited"], st["avg_particles_computed"],
                                     st["avg_monopoles_used"], st["total_operations"]])
    out["names"] = np.array(names)
    save("tree_statistics", **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["gauss10k", "small", "refit", "plummer1m", "statistics"]
    for w in which:
        t0 = time.time()
        {"gauss10k": case_gauss10k, "small": case_small, "refit": case_refit,
         "plummer1m": case_plummer_1m, "statistics": case_statistics}[w]()
        print(f"{w}: {time.time() - t0:.1f} s")
