"""Transform base class (src/pytomography/transforms/transform.py:8-38)."""
from __future__ import annotations

import abc


class Transform(metaclass=abc.ABCMeta):
    """Plugin applied inside a system matrix; ``configure`` receives the metadata."""

    def __init__(self) -> None:
        import pytomography_gb300 as _p
        self.device = _p.device

    def configure(self, object_meta, proj_meta) -> None:
        self.object_meta = object_meta
        self.proj_meta = proj_meta

    @abc.abstractmethod
    def forward(self, x, *args):
        ...

    @abc.abstractmethod
    def backward(self, x, *args):
        ...
