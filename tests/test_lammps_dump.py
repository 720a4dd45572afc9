"""LAMMPS dump text (dompap/tools/to_lammps_dump.py:4-48) against the
reference's own output (``tests/golden/lammps_ref.*``, written by
``make_golden.py --only lammps``): byte for byte from the same arrays on the
host, and from a GPU system restored from those arrays with the forces to
1e-10 relative RMS."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    g = dict(np.load(os.path.join(GOLDEN, "lammps_ref.npz")))
    with open(os.path.join(GOLDEN, "lammps_ref.txt")) as fh:
        text = fh.read()
    return g, text


def test_dump_text_is_byte_identical():
    from dompap_gb300.tools import to_lammps_dump

    g, text = _golden()
    stub = SimpleNamespace(number_of_steps=int(g["number_of_steps"]), box_vectors=g["box_vectors"],
                           positions=g["positions"], particle_types=g["particle_types"], masses=g["masses"],
                           image_positions=g["image_positions"], velocities=g["velocities"],
                           get_diameters=lambda: g["diameters"], get_forces=lambda: g["forces"])
    assert to_lammps_dump(stub) == text


def test_dump_rejects_other_dimensions_like_the_reference():
    from dompap_gb300.tools import to_lammps_dump

    with open(os.path.join(GOLDEN, "lammps_ref_2d_error.txt")) as fh:
        message = fh.read()
    stub = SimpleNamespace(number_of_steps=0, box_vectors=np.ones(2), positions=np.zeros((4, 2)))
    with pytest.raises(ValueError, match=message):
        to_lammps_dump(stub)


@pytest.mark.gpu
def test_dump_from_gpu_system():
    from dompap_gb300 import Simulation
    from dompap_gb300.tools import to_lammps_dump

    g, text = _golden()
    n = g["positions"].shape[0]
    sim = Simulation()
    sim.box_vectors = g["box_vectors"]
    sim.positions = g["positions"]
    sim.velocities = g["velocities"]
    sim.betas = np.zeros((n, 3))
    sim.image_positions = g["image_positions"]
    sim.masses = g["masses"]
    sim.particle_types = g["particle_types"]
    sim.set_pair_potential("4*(r**-12-r**-6)", 1.5)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=64)
    sim.number_of_steps = int(g["number_of_steps"])
    got = to_lammps_dump(sim).split("\n")
    want = text.split("\n")
    assert len(got) == len(want)
    assert got[:9] == want[:9]
    fg = np.array([[float(v) for v in line.split()[-3:]] for line in got[9:]])
    fw = np.array([[float(v) for v in line.split()[-3:]] for line in want[9:]])
    assert np.sqrt(np.mean((fg - fw) ** 2) / np.mean(fw ** 2)) <= 1e-10
    assert [line.split()[:-3] for line in got[9:]] == [line.split()[:-3] for line in want[9:]]
