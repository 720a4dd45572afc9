"""LAMMPS dump text of a system's state (dompap/tools/to_lammps_dump.py:4-48)."""
from __future__ import annotations

import numpy as np


def to_lammps_dump(sim) -> str:
    """Positions, images, velocities and forces (from the GPU) as LAMMPS dump
    text, with the reference's fields, order and number formatting (Python's
    shortest repr of each float64, ids from 0). As in the reference
    (dompap/tools/to_lammps_dump.py:22-28), only three dimensions are written:
    any other dimension raises ValueError('Dimension of space must be 2 or 3')."""
    number_of_steps = sim.number_of_steps
    box_vectors = np.asarray(sim.box_vectors)
    positions = np.asarray(sim.positions)
    dimension_of_space = positions.shape[1]
    number_of_atoms = positions.shape[0]
    head = ["ITEM: TIMESTEP\n", f"{number_of_steps:d}\n", f"ITEM: NUMBER OF ATOMS\n{number_of_atoms:d}\n"]
    if dimension_of_space != 3:
        raise ValueError("Dimension of space must be 2 or 3")
    head.append("ITEM: BOX BOUNDS pp pp pp\n")
    head.extend(f"0.0 {box_vectors[k]}\n" for k in range(3))
    head.append("ITEM: ATOMS id type diameter mass x y z ix iy iz vx vy vz fx fy fz")
    types = np.asarray(sim.particle_types).reshape(-1)
    masses = np.asarray(sim.masses).reshape(-1)
    diameters = np.asarray(sim.get_diameters()).reshape(-1)
    images = np.asarray(sim.image_positions)
    velocities = np.asarray(sim.velocities)
    forces = np.asarray(sim.get_forces())
    lines = []
    for n in range(number_of_atoms):
        x, v, f, im = positions[n], velocities[n], forces[n], images[n]
        lines.append(f"\n{n} {int(types[n])} {float(diameters[n])} {float(masses[n])} "
                     f"{x[0]} {x[1]} {x[2]} {int(im[0])} {int(im[1])} {int(im[2])} "
                     f"{v[0]} {v[1]} {v[2]} {f[0]} {f[1]} {f[2]}")
    return "".join(head) + "".join(lines)
