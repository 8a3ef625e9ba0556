"""Module-level tree stages (bhut/tree), on the GPU.

``TreeData`` comes from ``node``; ``build_tree``, ``refit_tree`` and
``should_refit_vs_rebuild`` are imported on first use (their modules use the
engine's API module, which itself imports ``TreeData`` from here).
"""
from .node import TreeData  # noqa: F401

_LAZY = {"build_tree": ".build", "refit_tree": ".refit", "should_refit_vs_rebuild": ".refit"}


def __getattr__(name):
    if name in _LAZY:
        import importlib
        return getattr(importlib.import_module(_LAZY[name], __name__), name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
