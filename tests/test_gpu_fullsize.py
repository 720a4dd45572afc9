"""The benchmark's own workloads at full size: 1,048,576 particles at density
1 with N(0, 0.01) jitter — fcc 64^3 (D = 3), the square lattice 1024^2 (D = 2)
and the hypercubic lattice 32^4 (D = 4) — (1-r)^2 with r_cut = 1, skin 0.2,
G-JF at T = 0.002, after 1000 steps. The neighbour rows of sampled particles
equal the oracle's double loop over all particles (bit-exact pair sets at the
list's reference positions), their forces equal the oracle's pair sums over
those rows (1e-10 relative RMS), and the whole force field conserves
momentum."""
import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu

R_CUT, SKIN = 1.0, 0.2
LATTICES = {
    2: (((0.0, 0.0),), (1024, 1024)),
    3: (None, (64, 64, 64)),  # fcc
    4: (((0.0, 0.0, 0.0, 0.0),), (32, 32, 32, 32)),
}


def _system(dim):
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC, generate_positions

    unit, cells = LATTICES[dim]
    unit = FCC if unit is None else unit
    rng = np.random.default_rng(2024)
    pos = generate_positions(unit, cells, (1.0,) * dim)
    box = np.array(cells, dtype=np.float64)
    scale = (pos.shape[0] / np.prod(box)) ** (1 / dim)
    box, pos = box * scale, pos * scale
    pos = pos + rng.normal(0.0, 0.01, size=pos.shape)
    img = np.floor(pos / box)
    pos = pos - img * box
    n = pos.shape[0]
    np.random.seed(2024)
    sim = Simulation()
    sim.box_vectors = box
    sim.positions = pos
    sim.velocities = rng.normal(0.0, np.sqrt(0.002), size=pos.shape)
    sim.betas = np.zeros_like(pos)
    sim.image_positions = img.astype(np.int32)
    sim.masses = np.ones((n, 1))
    sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    sim.set_pair_potential("(1-r)**2", R_CUT)
    sim.set_neighbor_list(skin=SKIN, max_number_of_neighbors=64, method_str="cell list")
    sim.set_integrator(time_step=0.01, target_temperature=0.002, temperature_damping_time=0.1)
    return sim


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_full_size_pair_sets_and_forces_against_oracle(dim):
    sim = _system(dim)
    sim.run(1000)
    n = sim.number_of_particles()
    assert n == 1048576
    box = np.array(sim.box_vectors)
    nl = np.array(sim.neighbor_list)
    ref_pos = np.array(sim.positions_neighbour_list)
    pos = np.array(sim.positions)
    forces = np.array(sim.get_forces())
    _, f_cut, _ = ref.make_pair_potential("(1-r)**2", R_CUT)
    cutoff = np.float64(1.0) * np.float64(R_CUT) + np.float64(SKIN)  # dompap/Simulation.py:353-356
    rng = np.random.default_rng(5)
    sample = rng.choice(n, size=200, replace=False)
    want_f = np.zeros((sample.size, dim))
    for k, i in enumerate(sample):
        # the pair set: get_neighbor_list_double_loop's test (dompap/neighbor_list.py:25-33) over all particles
        d = ref.displacement(ref_pos[i], ref_pos, box)
        r = np.sqrt(ref._sq_sum(d))
        mask = r < cutoff
        mask[i] = False
        row = nl[i][nl[i] >= 0]
        assert np.array_equal(row, np.nonzero(mask)[0]), i
        # the force of particle i over its row (dompap/potential.py:163-188)
        dd = ref.displacement(pos[i], pos[row], box)
        dist = ref._sq_sum(dd) ** 0.5
        want_f[k] = np.sum((f_cut(dist) / dist)[:, None] * dd, axis=0)
    got = forces[sample]
    scale = np.sqrt(np.mean(want_f ** 2))
    assert scale > 0.0  # the melted state has pairs inside r_cut
    assert np.sqrt(np.mean((got - want_f) ** 2)) <= 1e-10 * scale
    # pair forces are antisymmetric: the total vanishes to rounding
    assert np.all(np.abs(forces.sum(axis=0)) <= 1e-10 * np.abs(forces).sum(axis=0))
