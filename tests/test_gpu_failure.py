"""Failure detection without a GPU fault: a device-side wait that nothing
satisfies gives up after its iteration limit, frees the tensor memory it holds
and flags the failure; the host reports DP_ERR_TIMEOUT and the handle and
context stay usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable():
    from dompap_gb300 import Simulation
    from dompap_gb300 import _lib
    from dompap_gb300.positions import FCC

    np.random.seed(3)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=FCC, cells=(4, 4, 4), lattice_constants=(1, 1, 1))
    sim.set_masses(masses=1.0)
    sim.set_density(density=0.8)
    sim.set_pair_potential("4*(r**-12-r**-6)", 2.5)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=128)
    f0 = sim.get_forces()
    lib = _lib.load()
    for limit in (1, 256):
        rc = lib.dp_selftest_bounded_wait(sim._h, limit)
        assert rc == _lib.DP_ERR_TIMEOUT
        assert b"bounded device-side wait" in lib.dp_last_error()
    # the error was cleared and nothing else changed
    assert np.array_equal(sim.get_forces(), f0)
    sim.set_integrator(time_step=0.004, target_temperature=1.0, temperature_damping_time=0.1)
    sim.run(10)
    assert np.all(np.isfinite(sim.get_forces()))
