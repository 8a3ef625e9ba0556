"""bhut/tree/node.py: the TreeData container (host copy of a device tree)."""
from ..api import TreeData  # noqa: F401
