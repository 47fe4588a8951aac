"""Base metadata classes (src/pytomography/metadata/metadata.py:3-27)."""
from __future__ import annotations


class ObjectMeta:
    """Parent class of object-space metadata."""

    def __init__(self, dr, shape) -> None:
        self.dr = dr
        self.shape = shape


class ProjMeta:
    """Parent class of projection-space metadata."""

    def __init__(self, angles) -> None:
        self.angles = angles
