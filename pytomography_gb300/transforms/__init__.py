"""Transform (plugin) mirrors of ``src/pytomography/transforms``."""
from .transform import Transform  # noqa: F401
