"""Tools around ``Simulation`` (dompap/tools/__init__.py)."""

from .autotune import autotune  # noqa: F401
from .progress_bar import progress_bar  # noqa: F401
