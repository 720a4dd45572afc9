"""GPU integrators against the reference: the G-JF arithmetic with the device's
own normal deviates, deterministic trajectories (NVE leap-frog, G-JF with
tau = inf) against golden fixtures, wrap into box, the RNG's statistics and
dompap's doctest values."""
import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu


def _sim_from_traj(t, pot, r_cut, skin):
    from dompap_gb300 import Simulation

    sim = Simulation()
    n, d = t["positions0"].shape
    sim.box_vectors = t["box"]
    sim.positions = t["positions0"]
    sim.velocities = t["velocities0"]
    sim.betas = np.zeros((n, d))
    sim.image_positions = t["images0"]
    sim.masses = np.ones((n, 1))
    sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    sim.set_pair_potential(pot, r_cut)
    sim.set_neighbor_list(skin=skin, max_number_of_neighbors=256)
    return sim


def test_nve_trajectory(golden_traj):
    t = {k.split("/", 1)[1]: v for k, v in golden_traj.items() if k.startswith("nve/")}
    sim = _sim_from_traj(t, "4*(r**-12-r**-6)", 2.5, 0.3)
    sim.set_integrator(time_step=0.005)
    for _ in range(int(t["steps"])):
        sim.step_leap_frog()
    assert np.max(np.abs(sim.positions - t["positions"])) <= 1e-10
    assert np.max(np.abs(sim.velocities - t["velocities"])) <= 1e-9
    assert np.array_equal(sim.image_positions, t["images"])


def test_nve_trajectory_one_run_call(golden_traj):
    """The same 12 steps as one graph-replayed run."""
    t = {k.split("/", 1)[1]: v for k, v in golden_traj.items() if k.startswith("nve/")}
    sim = _sim_from_traj(t, "4*(r**-12-r**-6)", 2.5, 0.3)
    sim.set_integrator(time_step=0.005)
    sim.run_leap_frog(int(t["steps"]))
    assert np.max(np.abs(sim.positions - t["positions"])) <= 1e-10
    assert np.array_equal(sim.image_positions, t["images"])


def test_gjf_tau_inf_trajectory(golden_traj):
    t = {k.split("/", 1)[1]: v for k, v in golden_traj.items() if k.startswith("gjfinf/")}
    sim = _sim_from_traj(t, "(1-r)**2", 1.0, 0.2)
    sim.set_integrator(time_step=0.01, target_temperature=0.5, temperature_damping_time=np.inf)
    sim.run(int(t["steps"]))
    assert np.max(np.abs(sim.positions - t["positions"])) <= 1e-12
    assert np.max(np.abs(sim.velocities - t["velocities"])) <= 1e-12
    assert np.array_equal(sim.image_positions, t["images"])


def _d2f_trunc(x):
    """float64 -> float32 truncating the mantissa (the kernel's bit move)."""
    b = np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1023 + 127
    sign = ((b >> np.uint64(63)).astype(np.uint32)) << np.uint32(31)
    mant = ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    body = np.where(e <= 0, np.uint32(0),
                    np.where(e >= 255, np.uint32(0x7F800000),
                             (np.clip(e, 0, 255).astype(np.uint32) << np.uint32(23)) | mant))
    return (sign | body.astype(np.uint32)).view(np.float32)


@pytest.mark.parametrize("masses", ["classes", "one"])
def test_gjf_step_arithmetic(masses):
    """One G-JF step on the GPU equals make_one_step (dompap/integrator.py:17-40)
    fed with the GPU's own normal deviates for that step: the deterministic
    part a v + (b dt / m) F to float64 rounding, the noise terms
    beta_new = sqrt(2 alpha T dt) z and b (beta_old + beta_new) / (2m) exactly
    as their float32 products and sum."""
    from dompap_gb300 import Simulation
    from dompap_gb300 import _lib

    rng = np.random.default_rng(5)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0, 0, 0], [0.5, 0.5, 0.5]), cells=(5, 5, 5),
                      lattice_constants=(1, 1, 1))
    n = sim.number_of_particles()
    if masses == "classes":
        sim.set_masses(masses=list(rng.choice([1.0, 2.0, 0.5], size=n)))
    else:
        sim.set_masses(masses=1.5)
    sim.set_density(density=1.1)
    sim.positions = sim.positions + rng.normal(0, 0.05, size=sim.positions.shape)
    sim.wrap_into_box()
    sim.velocities = rng.normal(size=(n, 3))
    sim.betas = rng.normal(scale=0.1, size=(n, 3))
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=0.3)
    dt, temp, tau = 0.01, 0.7, 0.2
    sim.set_integrator(time_step=dt, target_temperature=temp, temperature_damping_time=tau)
    pos0, vel0, beta0 = np.array(sim.positions), np.array(sim.velocities), np.array(sim.betas)
    img0 = np.array(sim.image_positions)
    forces = sim.get_forces()
    step = int(sim._stats().steps)
    normals = np.empty((n, 3))
    _lib.check(_lib.load().dp_get_normals(sim._h, step, _lib.dptr(normals)))
    sim.step()
    m = np.array(sim.masses).reshape(n, 1)
    # the reference's coefficients (dompap/integrator.py:29-36)
    alpha = m / tau
    denominator = 1.0 + alpha * dt / 2.0 / m
    b = 1 / denominator
    c2 = (b / 2 / m).astype(np.float32)
    c3 = np.sqrt(2 * alpha * temp * dt).astype(np.float32)
    bn = c3 * normals.astype(np.float32)
    noise = c2 * (_d2f_trunc(beta0).reshape(n, 3) + bn)
    assert bn.dtype == np.float32 and noise.dtype == np.float32
    # deterministic part: make_one_step with both noise terms zero
    _, vel_det, _ = ref.gjf_step(pos0, vel0, np.zeros_like(beta0), forces, m, dt, temp, tau, np.zeros_like(normals))
    vel = vel_det + noise.astype(np.float64)
    pos = pos0 + vel * dt
    img = img0.copy()
    ref.wrap_into_box(pos, img, np.array(sim.box_vectors))
    assert np.array_equal(sim.betas, bn.astype(np.float64))
    assert np.max(np.abs(sim.velocities - vel)) <= 1e-13
    assert np.max(np.abs(sim.positions - pos)) <= 1e-13
    assert np.array_equal(sim.image_positions, img)


def test_normals_statistics():
    from dompap_gb300 import Simulation
    from dompap_gb300 import _lib

    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0, 0, 0],), cells=(40, 40, 40), lattice_constants=(1, 1, 1))
    sim.set_masses(masses=1.0)
    sim.set_pair_potential("(1-r)**2", 1.0)
    n = sim.number_of_particles()
    a = np.empty((n, 3))
    b = np.empty((n, 3))
    _lib.check(_lib.load().dp_get_normals(sim._h, 7, _lib.dptr(a)))
    _lib.check(_lib.load().dp_get_normals(sim._h, 8, _lib.dptr(b)))
    z = a.reshape(-1)
    assert abs(z.mean()) < 5 / np.sqrt(z.size)
    assert abs(z.var() - 1) < 5 * np.sqrt(2 / z.size)
    assert abs(np.mean(z ** 4) - 3) < 0.05
    assert abs(np.corrcoef(a.reshape(-1), b.reshape(-1))[0, 1]) < 5 / np.sqrt(z.size)
    c = np.empty((n, 3))
    _lib.check(_lib.load().dp_get_normals(sim._h, 7, _lib.dptr(c)))
    assert np.array_equal(a, c)


def test_wrap_into_box(golden_unit):
    from dompap_gb300 import Simulation

    sim = Simulation()
    sim.box_vectors = np.array([2.0, 2.0, 2.0])
    sim.positions = golden_unit["wrap/in"]
    sim.velocities = np.zeros((3, 3))
    sim.betas = np.zeros((3, 3))
    sim.image_positions = np.zeros((3, 3), dtype=np.int32)
    sim.masses = np.ones((3, 1))
    sim.particle_types = np.zeros((3, 1), dtype=np.int32)
    sim.wrap_into_box()
    assert np.array_equal(sim.positions, golden_unit["wrap/positions"])
    assert np.array_equal(sim.image_positions, golden_unit["wrap/images"])


def test_doctest_values(golden_unit):
    from dompap_gb300 import Simulation

    sim = Simulation()
    sim.scale_box(0.5)
    e = sim.get_potential_energy()
    assert abs(e - golden_unit["doctest/energy_scaled"]) <= 1e-12 * 167.06442443573454
    sim = Simulation()
    sim.positions[0] = [0.5, 0.0, 0.0]
    forces = sim.get_forces()
    # the float64-parity kernels agree with float64 to ~1e-14 relative (double-float
    # arithmetic on exact fixed-point displacements), not to the last bit
    assert abs(forces[0, 0] + 1.0) <= 1e-14 and forces[0, 1] == 0.0 and forces[0, 2] == 0.0
    sim = Simulation()
    assert abs(sim.get_laplacian()[0] - 12.0) <= 12.0 * 1e-14
    assert sim.number_of_particles() == 125
    assert f"{sim.get_density():.3f}" == "1.000"
    sim.set_density(density=0.9)
    assert f"{sim.get_density():.3f}" == "0.900"
    sim = Simulation()
    sim.set_random_velocities(temperature=0.0)
    assert sim.get_pressure() == 0.0
    assert sim.get_virial() == 0.0
    sim = Simulation()
    sim.set_integrator(time_step=0.01, target_temperature=1.0, temperature_damping_time=0.1)
    for _ in range(10):
        sim.step()
    assert sim.get_time() == 0.1
    sim.velocities = np.ones_like(sim.velocities)
    assert f"{sim.get_kinetic_energy():.1f}" == "187.5"
    # set_neighbor_list doctest (dompap/Simulation.py:327-333): a fresh system
    sim = Simulation()
    sim.set_neighbor_list()
    assert int(np.max(np.sum(sim.neighbor_list != -1, axis=1))) == 26


def test_copy_is_independent():
    from dompap_gb300 import Simulation

    sim = Simulation()
    cp = sim.copy()
    cp.positions[0] = [0.5, 0.0, 0.0]
    assert np.array_equal(sim.positions[:3], [[0, 0, 0], [0, 0, 1], [0, 0, 2]])
    assert np.array_equal(cp.positions[:3], [[0.5, 0, 0], [0, 0, 1], [0, 0, 2]])
    cp.run(5)
    assert np.array_equal(sim.positions[:1], [[0, 0, 0]])


def test_langevin_free_particle_temperature():
    """Non-interacting particles: the G-JF leap-frog velocities of
    dompap/integrator.py:37 have <m v^2> = T / (1 + dt / (2 tau)) per degree of
    freedom (stationary variance of that recursion); the GPU run reproduces it."""
    from dompap_gb300 import Simulation

    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0, 0, 0],), cells=(20, 20, 20), lattice_constants=(2, 2, 2))
    sim.set_masses(masses=1.0)
    sim.set_pair_potential("(1-r)**2", 0.05)
    sim.set_neighbor_list(skin=0.5, method_str="cell list")
    sim.set_integrator(time_step=0.01, target_temperature=0.5, temperature_damping_time=0.1)
    sim.run(500)
    temps = []
    for _ in range(40):
        sim.run(25)
        temps.append(sim.get_temperature())
    expected = 0.5 / (1 + 0.01 / (2 * 0.1))
    assert abs(np.mean(temps) - expected) < 0.004, (np.mean(temps), expected)


def _block_mean(x, nblocks=10):
    x = np.asarray(x)
    b = np.array_split(x, nblocks)
    m = np.array([v.mean() for v in b])
    return m.mean(), m.std(ddof=1) / np.sqrt(nblocks)


@pytest.mark.slow
def test_lj_ensemble_matches_oracle():
    """LJ fcc 500 at density 0.8442, T = 1 (the CPU-runnable case): ensemble
    means of T, U/N and P from the GPU run and from the oracle's own Langevin
    run agree within 4 combined standard errors (block averages), and so does
    g(r) bin by bin (5 standard errors, the first peak in the same bin)."""
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC

    rng = np.random.default_rng(21)
    np.random.seed(21)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=FCC, cells=(5, 5, 5), lattice_constants=(1, 1, 1))
    sim.set_masses(masses=1.0)
    sim.set_density(density=0.8442)
    sim.set_random_velocities(temperature=1.0)
    sim.set_pair_potential("4*(r**-12-r**-6)", 2.5)
    sim.set_neighbor_list(skin=0.5, max_number_of_neighbors=256)
    sim.set_integrator(time_step=0.005, target_temperature=1.0, temperature_damping_time=0.1)
    pos0, vel0, box = np.array(sim.positions), np.array(sim.velocities), np.array(sim.box_vectors)
    n = pos0.shape[0]
    equil, samples, stride = 600, 160, 10
    r_bins = np.linspace(0.0, 0.5 * float(box[0]), 61)
    sim.run(equil)
    g = {"T": [], "U": [], "P": [], "rdf": []}
    for _ in range(samples):
        sim.run(stride)
        g["T"].append(sim.get_temperature())
        g["U"].append(sim.get_potential_energy() / n)
        g["P"].append(sim.get_pressure())
        g["rdf"].append(sim.get_radial_distribution_function(r_bins)[1])
    o = ref.OracleSystem(pos0, vel0, np.ones(n), box, "4*(r**-12-r**-6)", 2.5, 0.5, max_neighbors=256)
    o.dt, o.temperature, o.damping_time = 0.005, 1.0, 0.1
    for _ in range(equil):
        o.step_gjf(rng.normal(size=(n, 3)))
    h = {"T": [], "U": [], "P": [], "rdf": []}
    for _ in range(samples):
        for _ in range(stride):
            o.step_gjf(rng.normal(size=(n, 3)))
        o.update_neighbor_list()
        t = float(np.sum(o.velocities ** 2) / (3 * n))
        h["T"].append(t)
        h["U"].append(ref.energy_neighbor_list(o.positions, box, o.u, o.nlist) / n)
        w = ref.virial_double_loop(o.positions, box, o.f)
        vol = float(np.prod(box))
        h["P"].append(w / vol + np.sum(o.velocities ** 2) / 3 / vol)
        h["rdf"].append(ref.radial_distribution_function(o.positions, o.positions, box, r_bins)[1])
    for key in ("T", "U", "P"):
        mg, eg = _block_mean(g[key])
        mo, eo = _block_mean(h[key])
        print(f"{key}: GPU {mg:.4f} +- {eg:.4f}   oracle {mo:.4f} +- {eo:.4f}")
        assert abs(mg - mo) < 4 * np.hypot(eg, eo) + 1e-3 * abs(mo), key
    # g(r): block means per bin
    blocks_g = np.array([b.mean(axis=0) for b in np.array_split(np.array(g["rdf"]), 10)])
    blocks_o = np.array([b.mean(axis=0) for b in np.array_split(np.array(h["rdf"]), 10)])
    mg, mo = blocks_g.mean(axis=0), blocks_o.mean(axis=0)
    err = np.hypot(blocks_g.std(axis=0, ddof=1), blocks_o.std(axis=0, ddof=1)) / np.sqrt(10)
    z = np.abs(mg - mo) / (err + 1e-3)
    # the first peak beyond the self pairs (dompap counts them, at r = 0)
    shell = 0.5 * (r_bins[1:] + r_bins[:-1]) > 0.5
    pg, po = np.argmax(np.where(shell, mg, 0.0)), np.argmax(np.where(shell, mo, 0.0))
    print(f"g(r): first peak GPU {mg[pg]:.3f} at bin {pg}, oracle {mo[po]:.3f} at bin {po}; "
          f"largest deviation {z.max():.2f} standard errors")
    assert pg == po and mg[pg] > 2.0
    assert z.max() < 5.0


def test_fp32_force_ensemble_matches_fp64():
    """The FP32-force mode (float32 pair forces, float64 integration and sums)
    samples the same Langevin ensemble as the float64-parity mode: T, U/N and
    P of a 4,000-particle LJ liquid within 4 combined standard errors."""
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC

    def ensemble(precision):
        np.random.seed(8)
        sim = Simulation(precision=precision)
        sim.set_positions(unit_cell_coordinates=FCC, cells=(10, 10, 10), lattice_constants=(1, 1, 1))
        sim.set_masses(masses=1.0)
        sim.set_density(density=0.8442)
        sim.set_random_velocities(temperature=1.2)
        sim.set_pair_potential("4*(r**-12-r**-6)", 2.5)
        sim.set_neighbor_list(skin=0.5, max_number_of_neighbors=256, method_str="cell list")
        sim.set_integrator(time_step=0.005, target_temperature=1.2, temperature_damping_time=0.1)
        n = sim.number_of_particles()
        sim.run(1000)
        obs = {"T": [], "U": [], "P": []}
        for _ in range(100):
            sim.run(20)
            obs["T"].append(sim.get_temperature())
            obs["U"].append(sim.get_potential_energy() / n)
            obs["P"].append(sim.get_pressure())
        return obs

    a, b = ensemble("fp64"), ensemble("fp32")
    for key in ("T", "U", "P"):
        ma, ea = _block_mean(a[key])
        mb, eb = _block_mean(b[key])
        print(f"{key}: fp64 {ma:.4f} +- {ea:.4f}   fp32 {mb:.4f} +- {eb:.4f}")
        assert abs(ma - mb) < 4 * np.hypot(ea, eb) + 1e-3 * abs(ma), key
