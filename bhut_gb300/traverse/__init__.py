"""Module-level traversal entry points (bhut/traverse), on the GPU."""
from .bh import (  # noqa: F401
    barnes_hut_accelerations,
    barnes_hut_accelerations_targets,
    compute_tree_statistics,
)
from .kernels import validate_kernel_inputs  # noqa: F401
