"""GPU parity with the reference: pair sets bit-exact, forces / energy / virial /
Laplacian within 1e-10 relative (FP64 mode), on the golden configurations
(produced by the unmodified reference) and on fresh seeded inputs checked by
the oracle.

Tolerances, FP64 mode: force relative RMS <= 1e-10; energy, virial within
1e-10 of the sum of absolute pair terms; Laplacian max error <= 1e-10 of its
largest magnitude. FP32-force mode: force relative RMS <= 1e-4 (stated per
configuration in the test output).
"""
import numpy as np
import pytest

from conftest import CONFIG_TAGS, config_of
from gpu_helpers import oracle_params, oracle_potential, rel_rms, sim_from_config
from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("method", ["double loop", "cell list"])
@pytest.mark.parametrize("tag", CONFIG_TAGS)
def test_golden_configuration(golden_configs, tag, method):
    cfg = config_of(golden_configs, tag)
    sim = sim_from_config(cfg, tag, method=method)
    pos, box = cfg["positions"], cfg["box"]
    # pair set, order and -1 padding as dompap's double loop
    nl = sim.neighbor_list
    k = cfg["nlist"].shape[1]
    assert np.all(nl[:, k:] == -1)
    assert np.array_equal(nl[:, :k], cfg["nlist"]), "pair set differs from the reference"
    forces = sim.get_forces()
    assert rel_rms(forces, cfg["forces"]) <= TOL
    u, f, c = oracle_potential(cfg, tag)
    sig, eps = oracle_params(cfg)
    onl = cfg["nlist"]
    if "energy" in cfg:
        scale = ref.pair_terms_abs_sum(pos, box, u, onl, sig, eps)
        assert abs(sim.get_potential_energy() - cfg["energy"]) <= TOL * max(scale, 1e-300)
    _, w_abs = ref.virial_double_loop(pos, box, f, sig, eps, return_abs=True)
    assert abs(sim.get_virial() - cfg["virial"]) <= TOL * max(w_abs, 1e-300)
    lap = sim.get_laplacian()
    assert np.max(np.abs(lap - cfg["laplacian"])) <= TOL * np.max(np.abs(cfg["laplacian"]))
    assert abs(sim.get_temperature() - cfg["temperature"]) <= 1e-12 * cfg["temperature"]
    assert abs(sim.get_kinetic_energy() - cfg["kinetic_energy"]) <= 1e-12 * cfg["kinetic_energy"]
    assert abs(sim.get_pressure() - cfg["pressure"]) <= TOL * (abs(cfg["pressure"]) + w_abs / sim.get_volume())
    if "rdf_g" in cfg:
        r, g = sim.get_radial_distribution_function(cfg["rdf_bins"])
        assert np.array_equal(r, cfg["rdf_r"])
        np.testing.assert_allclose(g, cfg["rdf_g"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("tag", ["lj500", "harm3d", "harm2d", "harm4d", "wahn", "expensive"])
def test_fp32_force_mode(golden_configs, tag):
    cfg = config_of(golden_configs, tag)
    sim = sim_from_config(cfg, tag, method="cell list", precision="fp32")
    forces = sim.get_forces()
    err = rel_rms(forces, cfg["forces"])
    print(f"{tag}: FP32-force relative RMS error {err:.2e}")
    assert err <= 1e-4
    assert np.array_equal(sim.neighbor_list[:, : cfg["nlist"].shape[1]], cfg["nlist"])


@pytest.mark.parametrize("dim,cells,density,seed", [(3, (6, 6, 6), 1.2, 1), (2, (30, 30), 1.1, 2),
                                                    (4, (6, 6, 6, 6), 1.3, 3)])
def test_fresh_inputs_against_oracle(dim, cells, density, seed):
    """Seeded random configurations (not from the fixtures): GPU vs oracle."""
    from dompap_gb300 import Simulation

    rng = np.random.default_rng(seed)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0.0] * dim,), cells=cells, lattice_constants=(1.0,) * dim)
    sim.set_masses(masses=1.0)
    sim.set_density(density=density)
    sim.positions = sim.positions + rng.normal(0, 0.05, size=sim.positions.shape)
    sim.wrap_into_box()
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=64, method_str="cell list")
    pos, box = np.array(sim.positions), np.array(sim.box_vectors)
    nl_ref, _ = ref.neighbor_list_double_loop(pos, box, 1.3, 64)
    assert np.array_equal(sim.neighbor_list, nl_ref)
    u, f, c = ref.make_pair_potential("(1-r)**2", 1.0)
    assert rel_rms(sim.get_forces(), ref.forces_neighbor_list(pos, box, f, nl_ref)) <= TOL
    e = ref.energy_neighbor_list(pos, box, u, nl_ref)
    assert abs(sim.get_potential_energy() - e) <= TOL * ref.pair_terms_abs_sum(pos, box, u, nl_ref)


def test_edge_cases_pair_set():
    """Reference unit-test geometry (tests/test_neighbor_list.py:12-51), an empty
    neighbourhood, coincident boundary values and positions outside the box."""
    from dompap_gb300 import Simulation

    sim = Simulation()
    sim.box_vectors = np.array([6.0, 6.0, 6.0])
    sim.positions = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [2, 2, 2], [5, 5, 0]], dtype=np.float64)
    sim.velocities = np.zeros((6, 3))
    sim.betas = np.zeros((6, 3))
    sim.image_positions = np.zeros((6, 3), dtype=np.int32)
    sim.masses = np.ones((6, 1))
    sim.particle_types = np.zeros((6, 1), dtype=np.int32)
    sim.set_pair_potential("(1-r)**2", 0.5)
    for method in ("double loop", "cell list"):
        sim.set_neighbor_list(skin=1.0, max_number_of_neighbors=4, method_str=method)
        assert np.array_equal(sim.neighbor_list, np.array([[1, 2, 3, 5], [0, 2, 3, -1], [0, 1, 3, -1],
                                                           [0, 1, 2, -1], [-1, -1, -1, -1], [0, -1, -1, -1]]))
    # positions left outside the box: the pair set follows the single-shift rule on raw coordinates
    raw = np.array([[0, 0, 0], [7, 0, 0], [0, -5.5, 0], [0, 0, 1], [2, 2, 2], [5, 5, 0]], dtype=np.float64)
    want, _ = ref.neighbor_list_double_loop(raw, np.array([6.0] * 3), 1.5, 8)
    for method in ("double loop", "cell list"):
        sim.positions = raw
        sim.set_neighbor_list(skin=1.0, max_number_of_neighbors=8, method_str=method)
        assert np.array_equal(sim.neighbor_list, want)


def test_overflow_grows_capacity():
    """max_number_of_neighbors set too small: dompap would write out of bounds;
    here the list capacity grows and the pair set stays complete."""
    from dompap_gb300 import Simulation

    rng = np.random.default_rng(11)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0.0, 0.0, 0.0],), cells=(8, 8, 8), lattice_constants=(1, 1, 1))
    sim.set_masses(masses=1.0)
    sim.set_density(density=1.0)
    sim.positions = sim.positions + rng.normal(0, 0.05, size=sim.positions.shape)
    sim.wrap_into_box()
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=0.6, max_number_of_neighbors=4, method_str="cell list")
    pos, box = np.array(sim.positions), np.array(sim.box_vectors)
    nl_ref, counts = ref.neighbor_list_double_loop(pos, box, 1.6, None)
    assert counts.max() > 4
    u, f, c = ref.make_pair_potential("(1-r)**2", 1.0)
    assert rel_rms(sim.get_forces(), ref.forces_neighbor_list(pos, box, f, nl_ref)) <= TOL
    sim.max_number_of_neighbors = np.int32(nl_ref.shape[1])
    assert np.array_equal(sim.neighbor_list, nl_ref)


def test_codegen_potential_values(golden_unit):
    """The NVRTC-compiled potential at sample points vs the reference's callables."""
    from dompap_gb300 import Simulation

    sim = Simulation()
    for tag, expr, rc in (("harm", "(1-r)**2", 1.0), ("lj", "4*(r**-12-r**-6)", 2.5),
                          ("exp", str(golden_unit["pot_exp/expr"]), 3.0)):
        sim.set_pair_potential(expr, rc)
        r = golden_unit[f"pot_{tag}/r"]
        for name, fn in (("u", sim.pair_potential), ("f", sim.pair_force), ("c", sim.pair_curvature)):
            want = golden_unit[f"pot_{tag}/{name}"]
            np.testing.assert_allclose(fn(r), want, rtol=1e-13, atol=1e-13 * np.max(np.abs(want)))
    sim.set_pair_potential("Harmonic repulsive")
    np.testing.assert_array_equal(sim.pair_potential(golden_unit["pot_hard/r"]), golden_unit["pot_hard/u"])
    assert sim.pair_potential(0.5) == 0.125


def test_bad_potential_raises():
    from dompap_gb300 import Simulation
    from dompap_gb300._lib import DompapGPUError

    sim = Simulation()
    with pytest.raises((ValueError, DompapGPUError, Exception)):
        sim.set_pair_potential("(1-r)**2 + x", 1.0)
    with pytest.raises(ValueError):
        sim.set_neighbor_list(method_str="bogus")
    with pytest.raises(ValueError):
        sim.set_pair_potential("(1-r)**2", 1.0, force_method="bogus")


@pytest.mark.parametrize("fused", ["1", "0"])
def test_far_positions_forces_and_steps(monkeypatch, fused):
    """Positions left far outside the box (beyond [-L/4, 5L/4), e.g. shifted by
    2 L): forces and the first steps follow the reference's single-shift
    arithmetic on the raw coordinates (the float64 fallback of the
    double-float pair loop and of the fused step); after the first step's wrap
    the next steps run the double-float path. NVE, against the oracle's step
    sequence (skin check -> forces -> leap-frog -> wrap)."""
    from dompap_gb300 import Simulation

    monkeypatch.setenv("DOMPAP_FUSED_STEP", fused)
    rng = np.random.default_rng(21)
    unit = ref.generate_positions(((0.0, 0.0, 0.0),), (4, 4, 4), (1.0, 1.0, 1.0))
    box = np.array([4.0, 4.0, 4.0]) * (64 / 0.7 / 64.0) ** (1 / 3)
    pos = unit * box / 4.0 + rng.normal(0, 0.03, size=unit.shape)
    pos[3, 0] += 2 * box[0]
    pos[17, 1] -= 3 * box[1]
    pos[40, 2] += box[2] * 1.6
    vel = rng.normal(0, 0.5, size=pos.shape)
    pot, rc, skin = "4*(r**-12-r**-6)", 1.5, 0.3
    sim = Simulation()
    sim.box_vectors = box
    sim.positions = pos
    sim.velocities = vel
    sim.betas = np.zeros_like(pos)
    sim.image_positions = np.zeros(pos.shape, dtype=np.int32)
    sim.masses = np.ones((64, 1))
    sim.particle_types = np.zeros((64, 1), dtype=np.int32)
    sim.set_pair_potential(pot, rc)
    sim.set_neighbor_list(skin=skin, max_number_of_neighbors=64, method_str="double loop")
    sim.set_integrator(time_step=0.002)
    o = ref.OracleSystem(pos, vel, np.ones((64, 1)), box, pot, rc, skin, max_neighbors=64)
    o.dt = 0.002
    assert rel_rms(sim.get_forces(), o.forces()) <= TOL
    for _ in range(3):
        o.step_leap_frog()
    sim.run_leap_frog(3)
    assert np.max(np.abs(sim.positions - o.positions)) <= 1e-11
    assert np.max(np.abs(sim.velocities - o.velocities)) <= 1e-10
    assert np.array_equal(sim.image_positions, o.images)
    assert rel_rms(sim.get_forces(), o.forces()) <= TOL


def _bare_sim(pos, box, vel=None):
    from dompap_gb300 import Simulation

    n, d = pos.shape
    sim = Simulation()
    sim.box_vectors = np.asarray(box, dtype=np.float64)
    sim.positions = pos
    sim.velocities = np.zeros((n, d)) if vel is None else vel
    sim.betas = np.zeros((n, d))
    sim.image_positions = np.zeros((n, d), dtype=np.int32)
    sim.masses = np.ones((n, 1))
    sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    return sim


def test_single_particle_and_pair_at_cut():
    """One particle: no pairs, zero force and energy, free flight through the
    box with its image counter. Two particles exactly r_cut apart: the pair is
    listed and its force is exactly zero (f(r_cut) = 0 for (1-r)^2)."""
    sim = _bare_sim(np.array([[0.5, 0.5, 0.5]]), [3.0, 3.0, 3.0], vel=np.array([[1.0, -2.0, 0.5]]))
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=0.2, max_number_of_neighbors=8)
    assert np.array_equal(sim.get_forces(), np.zeros((1, 3)))
    assert sim.get_potential_energy() == 0.0
    sim.set_integrator(time_step=0.05)
    o = ref.OracleSystem(np.array([[0.5, 0.5, 0.5]]), np.array([[1.0, -2.0, 0.5]]), np.ones((1, 1)),
                         np.array([3.0, 3.0, 3.0]), "(1-r)**2", 1.0, 0.2, max_neighbors=8)
    o.dt = 0.05
    for _ in range(100):  # 5 time units, through several images
        o.step_leap_frog()
    sim.run_leap_frog(100)
    assert np.array_equal(sim.positions, o.positions)
    assert np.array_equal(sim.image_positions, o.images)
    unwrapped = sim.positions + sim.image_positions * 3.0
    assert np.max(np.abs(unwrapped - (0.5 + 5.0 * np.array([1.0, -2.0, 0.5])))) <= 1e-12
    sim = _bare_sim(np.array([[0.25, 0.5, 0.5], [1.25, 0.5, 0.5]]), [3.0, 3.0, 3.0])
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=0.2, max_number_of_neighbors=8)
    assert np.array_equal(sim.neighbor_list, np.array([[1, -1, -1, -1, -1, -1, -1, -1],
                                                       [0, -1, -1, -1, -1, -1, -1, -1]]))
    assert np.array_equal(sim.get_forces(), np.zeros((2, 3)))


def test_non_cubic_box_forces_and_steps():
    """A strongly non-cubic box (per-axis fixed-point scales in the
    double-float pair loop): forces and NVE steps against the oracle."""
    rng = np.random.default_rng(31)
    spacing = np.array([1.06, 1.13, 1.15])
    cells = (5, 7, 4)
    box = spacing * np.array(cells)
    pos = ref.generate_positions(((0.0, 0.0, 0.0),), cells, tuple(spacing)) + rng.normal(0, 0.05, size=(140, 3))
    pos -= np.floor(pos / box) * box
    n = pos.shape[0]
    vel = rng.normal(0, 0.3, size=(n, 3))
    pot, rc, skin = "4*(r**-12-r**-6)", 2.0, 0.25
    sim = _bare_sim(pos, box, vel)
    sim.set_pair_potential(pot, rc)
    sim.set_neighbor_list(skin=skin, max_number_of_neighbors=96, method_str="cell list")
    sim.set_integrator(time_step=0.001)
    o = ref.OracleSystem(pos, vel, np.ones((n, 1)), box, pot, rc, skin, max_neighbors=96)
    o.dt = 0.001
    assert rel_rms(sim.get_forces(), o.forces()) <= TOL
    for _ in range(10):
        o.step_leap_frog()
    sim.run_leap_frog(10)
    assert np.max(np.abs(sim.positions - o.positions)) <= 1e-11
    assert np.array_equal(sim.image_positions, o.images)
    assert rel_rms(sim.get_forces(), o.forces()) <= TOL


def test_run_host_equals_setters_run_getters(golden_configs):
    """dp_run_host (host state in, steps, host state out in one call) gives
    bit-identical results to the separate setters, run and getters."""
    from dompap_gb300 import _lib

    cfg = config_of(golden_configs, "lj500")
    out = []
    for combined in (False, True):
        np.random.seed(77)
        sim = sim_from_config(cfg, "lj500", method="cell list")
        sim.set_integrator(time_step=0.004, target_temperature=1.2, temperature_damping_time=0.2)
        sim.run(5)
        lib, h = _lib.load(), sim._h
        n = sim.number_of_particles()
        rng = np.random.default_rng(3)
        pos = np.ascontiguousarray(np.array(sim.positions) + rng.normal(0, 1e-3, size=(n, 3)))
        vel = np.ascontiguousarray(rng.normal(0, 1.0, size=(n, 3)))
        beta = np.ascontiguousarray(rng.normal(0, 0.1, size=(n, 3)))
        p_out, v_out, b_out = np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3))
        if combined:
            _lib.check(lib.dp_run_host(h, _lib.dptr(pos), _lib.dptr(vel), _lib.dptr(beta), 7, _lib.DP_INT_GJF,
                                       _lib.dptr(p_out), _lib.dptr(v_out), _lib.dptr(b_out)))
        else:
            _lib.check(lib.dp_set_positions(h, _lib.dptr(pos)))
            _lib.check(lib.dp_set_velocities(h, _lib.dptr(vel)))
            _lib.check(lib.dp_set_betas(h, _lib.dptr(beta)))
            _lib.check(lib.dp_run(h, 7, _lib.DP_INT_GJF))
            _lib.check(lib.dp_get_positions(h, _lib.dptr(p_out)))
            _lib.check(lib.dp_get_velocities(h, _lib.dptr(v_out)))
            _lib.check(lib.dp_get_betas(h, _lib.dptr(b_out)))
        sim._mark_device_newer()
        out.append((p_out, v_out, b_out))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_cached_program_gives_the_same_forces(tmp_path):
    """A pair program loaded from the on-disk cubin cache in a second process
    gives bit-identical forces to the freshly compiled one."""
    import os
    import subprocess
    import sys

    script = (
        "import sys, numpy as np; sys.path.insert(0, %r)\n"
        "from dompap_gb300 import Simulation\n"
        "from dompap_gb300.positions import FCC\n"
        "sim = Simulation()\n"
        "sim.set_positions(unit_cell_coordinates=FCC, cells=(4, 4, 4), lattice_constants=(1, 1, 1))\n"
        "sim.set_masses(masses=1.0)\n"
        "sim.set_density(density=0.9)\n"
        "sim.positions = sim.positions + np.random.default_rng(1).normal(0, 0.03, sim.positions.shape)\n"
        "sim.set_pair_potential('4*(r**-12-r**-6) + 0.1*exp(-r)', 2.2)\n"
        "sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=128)\n"
        "np.save(sys.argv[1], sim.get_forces())\n"
    ) % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, DOMPAP_NVRTC_CACHE=str(tmp_path / "cache"))
    outs = []
    for k in range(2):
        out = tmp_path / f"f{k}.npy"
        subprocess.run([sys.executable, "-c", script, str(out)], env=env, check=True, timeout=600)
        outs.append(np.load(out))
    assert len(list((tmp_path / "cache").glob("*.dpcubin"))) >= 1
    assert np.array_equal(outs[0], outs[1])


def test_overflow_during_run_replays_the_chunk():
    """Particles converging on the box centre outgrow the list capacity inside
    a run(): the chunk is restored from its backup, the capacity grows and the
    chunk is replayed, ending bit-identical to a run that never overflowed."""
    from dompap_gb300 import Simulation

    def run(kmax):
        sim = Simulation()
        sim.set_positions(unit_cell_coordinates=([0.0, 0.0, 0.0],), cells=(8, 8, 8), lattice_constants=(1, 1, 1))
        sim.set_masses(masses=1.0)
        sim.set_density(density=1.0)
        box = np.array(sim.box_vectors)
        d = np.array(sim.positions) - 0.5 * box
        sim.velocities = -3.0 * d  # everything heads for the centre
        sim.set_pair_potential("(1-r)**2", 1.0)
        sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=kmax, method_str="cell list")
        sim.set_integrator(time_step=0.005)
        cap0 = int(sim._stats().neighbor_capacity)
        sim.run_leap_frog(120)
        st = sim._stats()
        return np.array(sim.positions), np.array(sim.velocities), int(st.neighbor_capacity), cap0, int(st.steps)

    pa, va, cap_a, cap0_a, steps_a = run(16)
    pb, vb, cap_b, _, steps_b = run(2048)
    assert steps_a == steps_b == 120
    assert cap0_a == 16 and cap_a > 16  # grew inside the run
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
