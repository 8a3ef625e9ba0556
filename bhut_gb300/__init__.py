"""bhut_gb300: a GB300-native (sm_103a) Barnes-Hut engine.

Drop-in for bhut 0.1.0's ``accelerations`` and ``Tree``: the tree build
(bounding box, Morton keys, stable radix sort, count-split topology, node
moments), refit and the softened monopole/P2P traversal run as hand-written
CUDA kernels in ``libbhut_gb300.so``, reached through the C ABI declared in
``include/bhut_gb300.h``.
"""
from .api import (  # noqa: F401
    DEFAULT_FORM,
    Tree,
    TreeData,
    accelerations,
    accelerations_chunks,
    build_tree,
    compute_tree_statistics,
    direct_accelerations,
    morton_argsort,
    morton_keys,
)

__version__ = "0.1.0"
__all__ = ["Tree", "accelerations"]
