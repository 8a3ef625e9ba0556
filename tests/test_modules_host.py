"""Host-side checks of the module-level functions mirroring bhut's module
paths (bhut.space.bbox, bhut.utils.morton, bhut.tree, bhut.traverse): the
argument errors the reference raises before any computation (no GPU)."""
import numpy as np
import pytest

from bhut_gb300.api import TreeData
from bhut_gb300.space import bbox
from bhut_gb300.traverse import kernels
from bhut_gb300.tree import build as tbuild
from bhut_gb300.tree import refit as trefit
from bhut_gb300.utils import morton


def test_bbox_argument_errors():
    with pytest.raises(ValueError, match="points must be 2D array"):
        bbox.aabb(np.zeros(5))
    with pytest.raises(ValueError, match="points array cannot be empty"):
        bbox.aabb(np.zeros((0, 3)))


def test_morton_argument_errors():
    with pytest.raises(ValueError, match="points01 must be 2D array"):
        morton.morton_codes(np.zeros(4))
    with pytest.raises(ValueError, match="points01 must have 2 or 3 dimensions, got 4"):
        morton.morton_codes(np.zeros((3, 4)))
    with pytest.raises(ValueError, match="points01 must have 2 or 3 dimensions"):
        morton.sort_by_morton(np.zeros((3, 1)))


def test_build_and_refit_argument_errors():
    with pytest.raises(ValueError, match="multipole must be 'mono'"):
        tbuild.build_tree(np.zeros((3, 3)), np.ones(3), dim=3, leaf_size=4, multipole="quad")
    with pytest.raises(ValueError, match="Cannot build tree with zero particles"):
        tbuild.build_tree(np.zeros((0, 3)), np.ones(0), dim=3, leaf_size=4)
    td = _tiny_tree()
    with pytest.raises(ValueError, match="new_positions has 3 particles but tree was built "
                                         "with 2 particles"):
        trefit.refit_tree(td, np.zeros((3, 3)), np.ones(3))
    with pytest.raises(ValueError, match="masses has 3 elements"):
        trefit.refit_tree(td, np.zeros((2, 3)), np.ones(3))
    with pytest.raises(ValueError, match="new_positions has 2 dimensions but tree has 3"):
        trefit.refit_tree(td, np.zeros((2, 2)), np.ones(2))
    # count or dimension changes: rebuild, decided on the host
    assert trefit.should_refit_vs_rebuild(td, np.zeros((3, 3))) is False
    assert trefit.should_refit_vs_rebuild(td, np.zeros((2, 2))) is False
    assert trefit.should_refit_vs_rebuild(td, np.zeros((2, 3)), boundary_check=False) is True


def test_validate_kernel_inputs_messages():
    v = kernels.validate_kernel_inputs
    with pytest.raises(ValueError, match="positions must be 2D array"):
        v(np.zeros(3), np.ones(3), 0.0)
    with pytest.raises(ValueError, match="masses must be 1D array"):
        v(np.zeros((3, 3)), np.ones((3, 1)), 0.0)
    with pytest.raises(ValueError, match="positions has 3 particles but masses has 2 elements"):
        v(np.zeros((3, 3)), np.ones(2), 0.0)
    with pytest.raises(ValueError, match="softening must be scalar or 1D array"):
        v(np.zeros((3, 3)), np.ones(3), np.ones((3, 1)))
    with pytest.raises(ValueError, match="softening array has 2 elements but need 3"):
        v(np.zeros((3, 3)), np.ones(3), np.ones(2))
    v(np.zeros((3, 3)), np.ones(3), np.full(3, 0.1))


def _tiny_tree():
    return TreeData(center=np.zeros((1, 3)), half_size=np.ones(1), mass=np.full(1, 2.0),
                    com=np.zeros((1, 3)), first_child=np.array([-1]), child_count=np.array([0]),
                    start=np.array([0]), count=np.array([2]), is_leaf=np.array([True]),
                    perm=np.array([1, 0]), dim=3, leaf_size=4)


def test_treedata_validate():
    td = _tiny_tree()
    td.validate()
    bad = _tiny_tree()
    bad.perm = np.array([0, 0])
    with pytest.raises(ValueError, match="perm is not a valid permutation"):
        bad.validate()
    bad = _tiny_tree()
    bad.count = np.array([3])
    with pytest.raises(ValueError, match="Root node count 3 != num_particles 2"):
        bad.validate()
    bad = _tiny_tree()
    bad.leaf_size = 1
    with pytest.raises(ValueError, match="Some leaf nodes exceed leaf_size"):
        bad.validate()
    bad = _tiny_tree()
    bad.com = np.zeros((2, 3))
    with pytest.raises(ValueError, match="com has shape"):
        bad.validate()
