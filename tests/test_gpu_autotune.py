"""``tools.autotune`` on the GPU (dompap/tools/autotune.py:4-178).

* The reference's own test (tests/test_autotune.py:5-29): fcc 4^3 at density
  0.8, (1-r)^2 with r_cut 1, started from skin 1.0; the tuned skin lies in
  (0.1, 1.9).
* The launch shapes the autotuner chooses between (one thread, four lanes or
  a warp per particle; 4 or 6 resident CTAs per SM) integrate the same
  trajectory: 20 NVE steps from one state agree within 1e-12 relative in
  float64 parity and 1e-6 with float32 pair forces (the lanes add their
  partial forces in another order; float32 rounding of ~1e-7 grows over the
  steps of an LJ liquid).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FCC = ((0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5))


def _reference_system():
    from dompap_gb300 import Simulation

    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=FCC, cells=(4, 4, 4), lattice_constants=(1.0, 1.0, 1.0))
    sim.set_density(density=0.8)
    sim.set_masses(masses=1.0)
    sim.set_random_velocities(temperature=1.0)
    sim.set_pair_potential(pair_potential_str="(1-r)**2", r_cut=1.0)
    sim.set_pair_potential_parameters(sigma=1.0, epsilon=1.0)
    sim.set_neighbor_list(skin=0.5, max_number_of_neighbors=128)
    sim.set_integrator(time_step=0.01, target_temperature=1.0, temperature_damping_time=0.1)
    sim.set_neighbor_list(skin=1.0, max_number_of_neighbors=512)
    return sim


def test_autotune_reference_case():
    from dompap_gb300.tools import autotune

    np.random.seed(2)
    sim = autotune(_reference_system(), steps=10)
    assert 0.1 < sim.neighbor_list_skin < 1.9, sim.neighbor_list_skin
    res = sim._autotune_results
    best = min(res["step_launch_times_s"], key=res["step_launch_times_s"].get)
    assert res["step_launch"] == best
    lanes, blocks = sim.get_step_launch()
    assert lanes == best[0] and lanes in (1, 4, 32)
    assert blocks in (4, 6)
    assert set(k[0] for k in res["step_launch_times_s"]) == {1, 4, 32}  # 256 particles: all three timed
    # dompap's force-method candidates: the list step and the double loop
    assert set(res["force_method_times_s"]) == {"neighbor list", "double loop"}
    assert sim.force_method_str == min(res["force_method_times_s"], key=res["force_method_times_s"].get)
    sim.run(200)
    assert np.all(np.isfinite(sim.positions))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_step_launch_shapes_agree(precision):
    from dompap_gb300 import Simulation

    np.random.seed(4)
    base = Simulation(precision=precision)
    base.set_positions(unit_cell_coordinates=FCC, cells=(6, 6, 6), lattice_constants=(1.0, 1.0, 1.0))
    base.set_density(density=0.8442)
    base.set_masses(masses=1.0)
    base.set_random_velocities(temperature=1.2)
    base.set_pair_potential("4*(r**-12-r**-6)", 2.5)
    base.set_neighbor_list(skin=0.4, max_number_of_neighbors=256, method_str="cell list")
    base.set_integrator(time_step=0.004, target_temperature=1.2, temperature_damping_time=0.1)
    base.run(50)
    pos0, vel0, img0 = np.array(base.positions), np.array(base.velocities), np.array(base.image_positions)
    out = {}
    for lanes in (1, 4, 32):
        for blocks in (4, 6):
            sim = base.copy()
            sim.positions, sim.velocities, sim.image_positions = pos0, vel0, img0
            sim.set_step_launch(lanes, blocks)
            assert sim.get_step_launch() == (lanes, blocks)
            sim.run_leap_frog(20)
            out[(lanes, blocks)] = np.array(sim.positions) + np.array(sim.image_positions) * np.array(sim.box_vectors)
    ref = out[(1, 4)]
    scale = np.max(np.abs(ref))
    tol = {"fp64": 1e-12, "fp32": 1e-6}[precision]
    for key, x in out.items():
        assert np.max(np.abs(x - ref)) <= tol * scale, key
