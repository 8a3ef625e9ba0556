"""Module-level tree stages (bhut/tree), on the GPU."""
from ..api import TreeData  # noqa: F401
from .build import build_tree  # noqa: F401
from .refit import refit_tree, should_refit_vs_rebuild  # noqa: F401
