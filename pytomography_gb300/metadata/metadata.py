"""Base metadata classes (src/pytomography/metadata/metadata.py:3-27)."""
from __future__ import annotations


class ObjectMeta:
    """Parent class of object-space metadata."""

    def __init__(self, dr, shape) -> None:
        self.dr = dr
        self.dx = dr[0]
        self.dy = dr[1]
        self.dz = dr[2]
        self.shape = shape


class ProjMeta:
    """Parent class of projection-space metadata."""

    def __init__(self, angles) -> None:
        self.angles = angles
        self.num_projections = len(angles)
