"""PET IO mirrors (``src/pytomography/io/PET``)."""
from . import shared  # noqa: F401
