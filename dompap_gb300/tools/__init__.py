"""Tools around ``Simulation`` (dompap/tools/__init__.py)."""

from .autotune import autotune  # noqa: F401
from .to_lammps_dump import to_lammps_dump  # noqa: F401
