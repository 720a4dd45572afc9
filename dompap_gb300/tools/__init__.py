"""Tools around ``Simulation`` (dompap/tools/__init__.py)."""

from .autotune import autotune  # noqa: F401
from .progress_bar import progress_bar  # noqa: F401
from .run_test_simulation import run_test_simulation  # noqa: F401
from .to_lammps_dump import to_lammps_dump  # noqa: F401
