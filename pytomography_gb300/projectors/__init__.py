"""System-matrix mirrors of ``src/pytomography/projectors``."""
from .system_matrix import SystemMatrix  # noqa: F401
