"""The fused step kernel (pair forces + integrate + wrap + skin test in one
launch, positions double-buffered) against the separate force and integrator
kernels: the same trajectory, G-JF and NVE, float64-parity and float32-force
modes, with chunk lengths that leave the positions in either buffer set."""
import numpy as np
import pytest

from gpu_helpers import config_of, sim_from_config

pytestmark = pytest.mark.gpu


def _trajectory(monkeypatch, golden_configs, tag, fused, precision, nve):
    monkeypatch.setenv("DOMPAP_FUSED_STEP", "1" if fused else "0")
    np.random.seed(1234)  # the Langevin seed is drawn when the Simulation is made
    cfg = config_of(golden_configs, tag)
    sim = sim_from_config(cfg, tag, method="cell list" if tag in ("lj500", "wahn") else "double loop",
                          precision=precision)
    if nve:
        sim.set_integrator(time_step=0.002)
        run = sim.run_leap_frog
    else:
        sim.set_integrator(time_step=0.004, target_temperature=1.2, temperature_damping_time=0.2)
        run = sim.run
    run(37)
    for _ in range(3):
        run(1)
    run(20)
    st = sim._stats()
    return (np.array(sim.positions), np.array(sim.velocities), np.array(sim.betas),
            np.array(sim.image_positions), int(st.steps))


@pytest.mark.parametrize("tag", ["lj500", "wahn", "harm2d", "harm4d"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nve", [False, True])
def test_fused_step_matches_separate_kernels(monkeypatch, golden_configs, tag, precision, nve):
    a = _trajectory(monkeypatch, golden_configs, tag, True, precision, nve)
    b = _trajectory(monkeypatch, golden_configs, tag, False, precision, nve)
    assert a[4] == b[4] == 60
    # the same operations, compiled once by NVRTC (fused) and once by nvcc
    # (separate kernel); for small systems the fused step splits each
    # particle's list over a warp, so its pair sums come in another order:
    # agreement to rounding (float32 sums in the FP32 mode), amplified over 60
    # steps
    tol = 1e-9 if precision == "fp64" else 1e-6
    assert np.max(np.abs(a[0] - b[0])) <= tol
    assert np.max(np.abs(a[1] - b[1])) <= 10 * tol
    assert np.max(np.abs(a[2] - b[2])) <= 10 * tol
    assert np.array_equal(a[3], b[3])


def test_fused_step_is_the_run_kernel(monkeypatch, golden_configs):
    """run() launches one pair kernel per step when fused: the fused step's
    last CTA sets the next step's rebuild condition, so only the first step of
    a graph chunk has the one-thread condition kernel (plus the step counter
    once per chunk and the list kernels of each rebuild)."""
    from dompap_gb300 import _lib

    monkeypatch.setenv("DOMPAP_FUSED_STEP", "1")
    cfg = config_of(golden_configs, "lj500")
    sim = sim_from_config(cfg, "lj500", method="cell list")
    sim.set_integrator(time_step=0.004, target_temperature=1.2, temperature_damping_time=0.2)
    sim.run(10)
    st0 = sim._stats()
    sim.run(64)  # one graph chunk (500 particles: chunks of up to 1024 steps)
    st1 = sim._stats()
    launches = int(_lib.load().dp_kernel_launches(sim._h))
    rebuilds = int(st1.rebuilds - st0.rebuilds)
    # list kernels per rebuild (+ the status kernel): the cell list's counting
    # sort (7), permutation into cell order (2) and build, or the all-pairs build
    per_rebuild = 11 if st1.method_used == _lib.DP_NL_CELL else 2
    if st1.conditional_graphs:
        # per step: dp_step; per chunk: one condition kernel and the step counter
        assert launches - 64 - per_rebuild * rebuilds == 2
    else:
        assert launches >= 64


def test_prepared_graphs_with_odd_chunks_match_split_runs():
    """run() captures every chunk graph it will launch before the first step,
    each keyed by the position buffer set current when it starts (a fused chunk
    of odd length leaves the other set current). 100,000 particles give chunks
    of 41 steps: run(100) = 41 + 41 + 18 must give the same trajectory, bit for
    bit, as run(41) followed by run(59) (the Langevin noise is keyed by step
    and particle id, and the list rebuilds happen at the same steps)."""
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC

    def system():
        np.random.seed(77)  # the same seed for the noise of both systems
        sim = Simulation()
        sim.set_positions(unit_cell_coordinates=FCC, cells=(25, 25, 40), lattice_constants=(1.0, 1.0, 1.0))
        sim.set_masses(masses=1.0)
        sim.set_density(density=1.0)
        rng = np.random.default_rng(5)
        sim.positions = sim.positions + rng.normal(0.0, 0.05, size=sim.positions.shape)
        sim.wrap_into_box()
        sim.velocities = rng.normal(0.0, 0.3, size=sim.positions.shape)
        sim.set_pair_potential("(1-r)**2", 1.0)
        sim.set_neighbor_list(skin=0.2, max_number_of_neighbors=64, method_str="cell list")
        sim.set_integrator(time_step=0.01, target_temperature=0.1, temperature_damping_time=0.1)
        return sim

    a, b = system(), system()
    assert a.number_of_particles() == 100000
    a.run(100)
    b.run(41)
    b.run(59)
    assert a._stats().rebuilds == b._stats().rebuilds
    assert np.array_equal(np.array(a.positions), np.array(b.positions))
    assert np.array_equal(np.array(a.velocities), np.array(b.velocities))
    assert np.array_equal(np.array(a.image_positions), np.array(b.image_positions))
