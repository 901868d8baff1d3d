"""Ranges containers of so3g.proj.ranges (python/proj/ranges.py)."""
from ..ranges import RangesInt32, RangesMatrix  # noqa: F401

Ranges = RangesInt32
