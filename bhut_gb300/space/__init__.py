"""Module-level bounding-box stages (bhut/space), on the GPU."""
from .bbox import aabb, normalize_to_unit  # noqa: F401
