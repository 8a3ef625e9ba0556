"""Module-level Morton stages (bhut/utils), on the GPU."""
from .morton import morton_codes, sort_by_morton  # noqa: F401
