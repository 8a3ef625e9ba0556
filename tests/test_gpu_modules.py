"""The module-level functions at the reference's module paths
(bhut_gb300.space.bbox, .utils.morton, .tree, .traverse) on the GPU, against
the reference's golden outputs."""
import numpy as np
import pytest

from bhut_gb300.space.bbox import aabb, normalize_to_unit
from bhut_gb300.traverse.bh import (barnes_hut_accelerations, barnes_hut_accelerations_targets,
                                    compute_tree_statistics)
from bhut_gb300.tree.build import build_tree
from bhut_gb300.tree.refit import refit_tree, should_refit_vs_rebuild
from bhut_gb300.utils.morton import morton_codes, sort_by_morton
from conftest import TREE_FIELDS, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    yield


def _numpy_unit(pos, lo, hi, eps=1e-12):
    extent = hi - lo
    ext = np.where(extent <= 0, 1.0, extent)
    off = np.where(extent <= 0, 0.5, 0.0)
    return np.minimum((pos - lo) / ext + off, 1.0 - eps)


def _equal_tree(td, g, prefix):
    for f in TREE_FIELDS:
        a = np.asarray(getattr(td, f))
        assert np.array_equal(a.astype(g[prefix + f].dtype), g[prefix + f]), prefix + f


def test_stages_match_reference(golden_small):
    g = golden_small
    for name in g["names"]:
        pos, m = g[f"{name}__pos"], g[f"{name}__masses"]
        lo, hi = aabb(pos)
        assert np.array_equal(lo, pos.min(0)) and np.array_equal(hi, pos.max(0))
        p01 = normalize_to_unit(pos, lo, hi)
        assert np.array_equal(p01, _numpy_unit(pos, lo, hi)), name
        assert np.array_equal(morton_codes(p01), g[f"{name}__keys"]), name
        codes, perm, [sm] = sort_by_morton(p01, [m])
        assert np.array_equal(perm, g[f"{name}__L32__perm"]), name
        assert np.array_equal(codes, np.sort(g[f"{name}__keys"], kind="stable")), name
        assert np.array_equal(sm, m[perm]), name
        for L in (1, 32):
            td = build_tree(pos, m, dim=pos.shape[1], leaf_size=L, xp=None)
            _equal_tree(td, g, f"{name}__L{L}__")
            td.validate()


def test_morton_bits_and_range_errors():
    rng = np.random.default_rng(1)
    p = rng.random((1000, 3))
    for bits in (4, 10, 21):
        q = np.minimum((p * (1 << bits)).astype(np.uint64), (1 << bits) - 1)
        x = _expand3(q[:, 0]) | (_expand3(q[:, 1]) << np.uint64(1)) | (_expand3(q[:, 2]) << np.uint64(2))
        assert np.array_equal(morton_codes(p, bits), x), bits
    with pytest.raises(ValueError, match=r"All points must be in range \[0, 1\)"):
        morton_codes(np.array([[0.5, 1.0, 0.2]]))
    with pytest.raises(ValueError, match="Data array has 3 elements but need 1000"):
        sort_by_morton(p, [np.ones(3)])
    # data arrays of any row shape and dtype are permuted on the device
    extra = rng.integers(0, 100, (1000, 2, 3)).astype(np.int16)
    _, perm, [e] = sort_by_morton(p, [extra])
    assert np.array_equal(e, extra[perm])


def _expand3(x):
    x = x.astype(np.uint64)
    for sh, mask in ((32, 0x1F00000000FFFF), (16, 0x1F0000FF0000FF), (8, 0x100F00F00F00F00F),
                     (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249)):
        x = (x | (x << np.uint64(sh))) & np.uint64(mask)
    return x


@pytest.mark.parametrize("form", ["exact", "fast"])
def test_refit_and_traverse_modules(golden_refit, form):
    g = golden_refit
    tol = 1e-12 if form == "exact" else 1e-11
    for tag, L in (("plain", 16), ("negmass", 16)):
        pos, m = g[f"{tag}__pos"], g[f"{tag}__masses"]
        pos2, m2 = g[f"{tag}__pos2"], g[f"{tag}__masses2"]
        td = build_tree(pos, m, dim=3, leaf_size=L, xp=None)
        assert should_refit_vs_rebuild(td, pos2)
        tr = refit_tree(td, pos2, m2, None)
        _equal_tree(tr, g, f"{tag}__refit__")
        idx = g[f"{tag}__sample"]
        acc = barnes_hut_accelerations(tr, pos2, m2, 0.01, 0.5, 1.0, form=form)
        assert rel_l2(acc[idx], g[f"{tag}__acc"]) <= tol, tag
    td = build_tree(g["moved__pos"], g["moved__masses"], dim=3, leaf_size=8)
    assert not should_refit_vs_rebuild(td, g["moved__pos3"])


def test_targets_and_statistics_modules(golden_small, oracle_mod):
    g = golden_small
    for name in ("normal_n257", "zero_masses_n50", "normal2d_n300"):
        pos, m = g[f"{name}__pos"], g[f"{name}__masses"]
        td = build_tree(pos, m, dim=pos.shape[1], leaf_size=4)
        tg = g[f"{name}__targets"]
        a = barnes_hut_accelerations_targets(td, pos, m, tg, 0.01, theta=0.7, form="exact")
        assert rel_l2(a, g[f"{name}__L4__t0.7__e0.01__ext"]) <= 1e-12, name
        st = compute_tree_statistics(td, pos, 0.5)
        ot = oracle_mod.build_tree(pos, m, 4)
        nodes, parts, monos = oracle_mod.tree_statistics(ot, pos, 0.5)
        assert st["total_operations"] == parts + monos


def test_aabb_infinities_nan_and_signed_zero_like_numpy():
    """aabb (bbox.py:14-46) on values the integer-image min/max must order
    like numpy: infinities, NaN (propagates to its axis) and signed zeros."""
    rng = np.random.default_rng(13)
    pts = rng.standard_normal((5000, 3))
    pts[17, 0] = np.inf
    pts[4000, 0] = -np.inf
    pts[123, 1] = np.nan
    pts[:, 2] = np.where(rng.random(5000) < 0.5, 0.0, -0.0)
    lo, hi = aabb(pts)
    with np.errstate(invalid="ignore"):
        ref_lo, ref_hi = pts.min(0), pts.max(0)
    assert lo[0] == -np.inf and hi[0] == np.inf
    assert np.isnan(lo[1]) and np.isnan(hi[1])
    assert lo[2] == 0.0 and hi[2] == 0.0   # -0.0 == 0.0, as numpy's
    np.testing.assert_array_equal(lo, ref_lo)
    np.testing.assert_array_equal(hi, ref_hi)
    # finite inputs in 1-D and 2-D: exact extrema
    for d in (1, 2):
        q = rng.standard_normal((3001, d)) * 1e3
        lo, hi = aabb(q)
        assert np.array_equal(lo, q.min(0)) and np.array_equal(hi, q.max(0))
