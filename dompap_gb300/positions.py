"""Host-side lattice set-up (not on the per-step path).

``generate_positions`` builds the same lattice, in the same particle order, as
dompap/positions.py:33-52: cell index in C order (last axis fastest), the
basis particles of each cell consecutive, then scaled by the lattice constants.
"""
from __future__ import annotations

import numpy as np


def generate_positions(unit_cell_coordinates, cells, lattice_constants) -> np.ndarray:
    """Lattice positions, cells in row-major order and the unit cell's sites
    within each (dompap/positions.py:33-52)."""
    unit = np.asarray(unit_cell_coordinates, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int64)
    lat = np.asarray(lattice_constants, dtype=np.float64)
    n_cells = int(np.prod(cells))
    grid = np.indices(tuple(int(c) for c in cells), dtype=np.float64).reshape(len(cells), n_cells).T
    pos = (grid[:, None, :] + unit[None, :, :]).reshape(n_cells * unit.shape[0], unit.shape[1])
    pos *= lat
    return np.ascontiguousarray(pos)


FCC = ((0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5))
