"""dompap's force and energy method strings on the GPU
(dompap/Simulation.py:126-133, get_forces :594-654, get_potential_energy
:545-592): the neighbour-list kernels and the all-pairs kernels that stand in
for the double-loop and vectorised methods (dompap/potential.py:103-160,
191-250, 298-324), against the reference's own outputs for every method on
the golden configurations (``golden_methods.npz``), including an asymmetric
epsilon(n, m), where "double loop single core" and the double-loop energies
differ from the list sums. Then a system large enough for the cell list (its
state permuted into cell order) with an asymmetric dense epsilon: virial and
double-loop energy against the oracle (the upper-triangle sums follow particle
ids, not slots), and a run with the all-pairs step against a run with the list
step. Tolerances as in test_gpu_parity: forces 1e-10 relative RMS, energies
1e-10 of the sum of absolute pair terms."""
import numpy as np
import pytest

from conftest import config_of, load_golden
from gpu_helpers import oracle_params, oracle_potential, rel_rms, sim_from_config
from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu
TOL = 1e-10
FORCE_METHODS = ("neighbor list", "double loop", "double loop single core", "vectorized")
ENERGY_METHODS = ("neighbor list", "double loop", "double loop single core")


@pytest.mark.parametrize("tag", ["callable", "wahn", "harm2d"])
def test_methods_match_the_reference(golden_configs, tag):
    gold = load_golden("golden_methods.npz")
    cfg = config_of(golden_configs, tag)
    sim = sim_from_config(cfg, tag, method="cell list")
    pos, box = cfg["positions"], cfg["box"]
    u, f, _ = oracle_potential(cfg, tag)
    sig, eps = oracle_params(cfg)
    nl, _ = ref.neighbor_list_double_loop(pos, box, np.max(sig) * float(cfg["r_cut"]) + float(cfg["skin"]))
    scale = ref.pair_terms_abs_sum(pos, box, u, nl, sig, eps)
    for method in FORCE_METHODS:
        sim.force_method_str = method
        got = sim.get_forces()
        assert rel_rms(got, gold[f"{tag}/forces/{method}"]) <= TOL, method
    for method in ENERGY_METHODS:
        sim.energy_method_str = method
        assert abs(sim.get_potential_energy() - gold[f"{tag}/energy/{method}"]) <= TOL * scale, method


def _asymmetric_system():
    from dompap_gb300 import Simulation

    np.random.seed(12)
    sim = Simulation()
    fcc = ((0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5))
    sim.set_positions(unit_cell_coordinates=fcc, cells=(8, 8, 8), lattice_constants=(1.0, 1.0, 1.0))
    sim.set_masses(masses=1.0)
    sim.set_density(density=1.3)
    rng = np.random.default_rng(12)
    sim.positions = sim.positions + rng.normal(0.0, 0.05, size=sim.positions.shape)
    sim.wrap_into_box()
    n = sim.number_of_particles()
    eps_m = 1.0 + 0.01 * (np.arange(n)[:, None] % 5) + 0.003 * (np.arange(n)[None, :] % 7)  # eps(n, m) != eps(m, n)
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_pair_potential_parameters(sigma=1.0, epsilon=lambda a, b: eps_m[a, b])
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=64, method_str="cell list")
    sim.set_integrator(time_step=0.005, target_temperature=0.5, temperature_damping_time=0.2)
    return sim, eps_m


def test_upper_triangle_sums_follow_particle_ids():
    sim, eps_m = _asymmetric_system()
    sim.run(200)  # rebuilds permute the state into cell order
    st = sim._stats()
    assert st.method_used == 0 and st.cells[0] >= 3 and st.rebuilds >= 2  # cell list, permuted
    pos, box = np.array(sim.positions), np.array(sim.box_vectors)
    u, f, _ = ref.make_pair_potential("(1-r)**2", 1.0)
    w, w_abs = ref.virial_double_loop(pos, box, f, 1.0, eps_m, return_abs=True)
    assert abs(sim.get_virial() - w) <= TOL * w_abs
    nl, _ = ref.neighbor_list_double_loop(pos, box, 1.3)
    scale = ref.pair_terms_abs_sum(pos, box, u, nl, 1.0, eps_m)
    sim.energy_method_str = "double loop"
    assert abs(sim.get_potential_energy() - ref.energy_double_loop(pos, box, u, 1.0, eps_m)) <= TOL * scale
    sim.energy_method_str = "neighbor list"
    assert abs(sim.get_potential_energy() - ref.energy_neighbor_list(pos, box, u, nl, 1.0, eps_m)) <= TOL * scale
    sim.force_method_str = "double loop single core"
    want = ref.forces_double_loop_single_core(pos, box, f, 1.0, eps_m)
    assert rel_rms(sim.get_forces(), want) <= TOL
    sim.force_method_str = "neighbor list"
    assert rel_rms(sim.get_forces(), ref.forces_neighbor_list(pos, box, f, nl, 1.0, eps_m)) <= TOL


def test_allpairs_step_follows_the_list_step():
    """NVE from one state: the all-pairs step (no list kept) and the list step
    give the same trajectory within float64 rounding of the pair sums."""
    a, _ = _asymmetric_system()
    a.run(50)
    b = a.copy()
    b.force_method_str = "double loop"
    for sim in (a, b):
        sim.run_leap_frog(30)
    xa = np.array(a.positions) + np.array(a.image_positions) * np.array(a.box_vectors)
    xb = np.array(b.positions) + np.array(b.image_positions) * np.array(b.box_vectors)
    assert np.max(np.abs(xa - xb)) <= 1e-11 * np.max(np.abs(xa))
