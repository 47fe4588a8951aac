"""Metadata mirrors of ``src/pytomography/metadata`` for the projector hot path."""
from .metadata import ObjectMeta, ProjMeta  # noqa: F401
