"""Batched replicas (one persistent kernel for many systems): float32 forces
against the float64 oracle per replica (relative RMS <= 1e-4), the integrator
against the single-system path, ensemble means against single-system runs, and
the launch autotuner."""
import numpy as np
import pytest

from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu
LJ = "4*(r**-12-r**-6)"


def small_specs(seed=3, n_rep=24):
    from dompap_gb300.batched import lj_replica_specs

    return lj_replica_specs(n_rep=n_rep, seed=seed, n_min=100, n_max=2500)


def test_batched_forces_match_fp64_oracle():
    from dompap_gb300.batched import Replicas

    specs, _ = small_specs()
    reps = Replicas(specs, LJ, 2.5, time_step=0.005, damping_time=0.1, seed=1)
    pos0, _, _ = reps.state()
    reps.run(1, record_forces=True)
    forces = reps.last_forces()
    u, f, c = ref.make_pair_potential(LJ, 2.5)
    worst = 0.0
    for r in range(reps.n_rep):
        sl = reps.replica_slice(r)
        p = pos0[sl]
        nl, _ = ref.neighbor_list_double_loop(p, reps.boxes[r], 2.5, None)
        want = ref.forces_neighbor_list(p, reps.boxes[r], f, nl)
        err = np.sqrt(np.mean((forces[sl] - want) ** 2) / np.mean(want ** 2))
        worst = max(worst, err)
    print(f"worst replica force relative RMS error (float32 vs oracle float64): {worst:.2e}")
    assert worst <= 1e-4


def test_batched_step_matches_single_system():
    """A deterministic NVE step of one replica equals the single-system FP32
    path on the same state (same float32 forces up to summation order)."""
    from dompap_gb300 import Simulation
    from dompap_gb300.batched import Replicas

    specs, _ = small_specs(seed=5, n_rep=6)
    reps = Replicas(specs, LJ, 2.5, time_step=0.005, seed=2)
    pos0, vel0, _ = reps.state()
    reps.run(5, nve=True)
    pos1, vel1, img1 = reps.state()
    for r in (0, 3):
        sl = reps.replica_slice(r)
        sim = Simulation(precision="fp32")
        n = sl.stop - sl.start
        sim.box_vectors = reps.boxes[r]
        sim.positions = pos0[sl]
        sim.velocities = vel0[sl]
        sim.betas = np.zeros((n, 3))
        sim.image_positions = np.zeros((n, 3), dtype=np.int32)
        sim.masses = np.ones((n, 1))
        sim.particle_types = np.zeros((n, 1), dtype=np.int32)
        sim.set_pair_potential(LJ, 2.5)
        sim.set_neighbor_list(skin=0.3, method_str="cell list")
        sim.set_integrator(time_step=0.005)
        sim.run_leap_frog(5)
        unwrapped_gpu = pos1[sl] + img1[sl] * reps.boxes[r]
        unwrapped_sim = np.asarray(sim.positions) + np.asarray(sim.image_positions) * reps.boxes[r]
        assert np.max(np.abs(unwrapped_gpu - unwrapped_sim)) < 1e-5
        assert np.max(np.abs(vel1[sl] - np.asarray(sim.velocities))) < 1e-4


def test_batched_ensemble_matches_single_system():
    """Langevin means of U/N and T per replica agree with the single-system
    float64 path within 4 combined standard errors."""
    from dompap_gb300 import Simulation
    from dompap_gb300.batched import Replicas, ReplicaSpec, fcc_cells_for
    from dompap_gb300.positions import FCC, generate_positions

    rng = np.random.default_rng(11)
    lat = (4 / 0.8442) ** (1 / 3)
    specs = []
    for n_target, temp in ((500, 1.0), (864, 1.6)):
        cells = fcc_cells_for(n_target)
        box = np.array(cells, float) * lat
        pos = generate_positions(FCC, cells, (lat,) * 3)
        specs.append(ReplicaSpec(pos, rng.normal(0, np.sqrt(temp), pos.shape), box, temp))
    reps = Replicas(specs, LJ, 2.5, time_step=0.005, damping_time=0.1, seed=4)
    reps.run(1000)
    blocks = {"U": [], "T": []}
    for _ in range(10):
        reps.run(200, sample_every=10)
        o = reps.observables(reset=True)
        blocks["U"].append(o["potential_energy_per_particle"])
        blocks["T"].append(o["temperature"])
    for r, spec in enumerate(specs):
        np.random.seed(100 + r)
        sim = Simulation()
        n = spec.positions.shape[0]
        sim.box_vectors = spec.box
        sim.positions = spec.positions
        sim.velocities = spec.velocities
        sim.betas = np.zeros((n, 3))
        sim.image_positions = np.zeros((n, 3), dtype=np.int32)
        sim.masses = np.ones((n, 1))
        sim.particle_types = np.zeros((n, 1), dtype=np.int32)
        sim.set_pair_potential(LJ, 2.5)
        sim.set_neighbor_list(skin=0.5, method_str="cell list")
        sim.set_integrator(time_step=0.005, target_temperature=spec.temperature, temperature_damping_time=0.1)
        sim.run(1000)
        su, st = [], []
        for _ in range(10):
            u_b, t_b = [], []
            for _ in range(20):
                sim.run(10)
                u_b.append(sim.get_potential_energy() / n)
                t_b.append(sim.get_temperature())
            su.append(np.mean(u_b))
            st.append(np.mean(t_b))
        for key, single in (("U", su), ("T", st)):
            b = np.array([x[r] for x in blocks[key]])
            s = np.array(single)
            err = np.hypot(b.std(ddof=1), s.std(ddof=1)) / np.sqrt(len(b))
            print(f"replica {r} {key}: batched {b.mean():.4f} single {s.mean():.4f} (+- {err:.4f})")
            # 10 blocks give a noisy standard error (the batched run's cell
            # binning orders float32 sums by atomics, so each run samples a
            # different trajectory): 5 of them plus 0.1 %
            assert abs(b.mean() - s.mean()) < 5 * err + 1e-3 * abs(s.mean())


def test_batched_autotune_and_full_shape():
    from dompap_gb300.batched import Replicas

    specs, rejected = small_specs(seed=9, n_rep=64)
    reps = Replicas(specs, LJ, 2.5, seed=3)
    best, ms = reps.autotune(steps=5, candidates=[(512, 128, 512), (1024, 256, 1024)])
    assert best in [(512, 128, 512), (1024, 256, 1024)]
    assert ms > 0
    pos, vel, img = reps.state()
    assert np.all(np.isfinite(pos)) and np.all(pos >= 0)
    for r in range(reps.n_rep):
        assert np.all(pos[reps.replica_slice(r)] <= reps.boxes[r])


def _run_batch(skin, kmax=0, steps=30, seed=4):
    from dompap_gb300.batched import Replicas

    specs, _ = small_specs(seed=seed, n_rep=12)
    reps = Replicas(specs, LJ, 2.5, time_step=0.005, damping_time=0.1, seed=9, skin=skin,
                    max_number_of_neighbors=kmax)
    reps.run(steps)
    pos, vel, img = reps.state()
    return pos, vel, img, reps.list_stats()


def test_batched_lists_match_stencil():
    """Verlet lists (rebuilt on the skin test) and the 27-cell stencil every
    step give the same trajectory: the same pairs, float32 sums in another order."""
    pa, va, ia, st = _run_batch(0.3)
    pb, vb, ib, _ = _run_batch(-1.0)
    assert st["builds"] >= 12 and st["overflowed"] == 0 and st["kmax"] > 0
    assert np.array_equal(ia, ib)
    assert np.max(np.abs(pa - pb)) <= 1e-4
    assert np.max(np.abs(va - vb)) <= 1e-3


def test_batched_list_overflow_falls_back_to_stencil():
    """A list capacity far below the pair count: every replica's first build
    overflows, is counted, and the replica uses the stencil (no pair lost)."""
    pa, va, ia, st = _run_batch(0.3, kmax=8, steps=10)
    pb, vb, ib, _ = _run_batch(-1.0, steps=10)
    assert st["overflowed"] == 12 and st["kmax"] == 8
    assert np.max(np.abs(pa - pb)) <= 1e-5
