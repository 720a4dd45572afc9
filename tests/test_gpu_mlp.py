"""Pair surrogate (tensor-core MLP): the GPU forward and gradients against the
float64 NumPy oracle of the same network, training on samples of the
generated float64 kernel, and the surrogate in the force/energy kernels
against that kernel (force relative RMS error, NVE energy drift, speed)."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu

EXPENSIVE_RAW = "4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r)"


def expensive_string(r_cut=3.0):
    import sympy as sp

    r = sp.symbols("r")
    u = sp.sympify(EXPENSIVE_RAW)
    u_rc = float(sp.N(u.subs(r, r_cut), 30))
    du_rc = float(sp.N(sp.diff(u, r).subs(r, r_cut), 30))
    return f"{EXPENSIVE_RAW} - ({u_rc!r}) - (r - {float(r_cut)!r})*({du_rc!r})"


@pytest.fixture(scope="module")
def surrogate():
    from dompap_gb300.mlp import PairSurrogate

    sur = PairSurrogate(expensive_string(), 3.0, r_min=0.8, n_samples=2 ** 20, seed=0)
    # ranked on a small lattice of another noise seed than the target test's
    starts = sur.fit(steps=100000, restarts=3, rank_on=_jittered_fcc((16, 16, 16), seed=7), batch=16384, lr0=2e-3,
                     lr1=1e-6)
    print("force errors of the starts on the ranking lattice:", starts)
    return sur


def test_forward_and_gradients_match_oracle():
    from dompap_gb300.mlp import PairSurrogate

    sur = PairSurrogate(expensive_string(), 3.0, n_samples=4096, seed=5)
    rng = np.random.default_rng(2)
    p = rng.normal(0, 0.3, sur.nparam).astype(np.float32)
    sur.set_params(p)
    r = rng.uniform(0.8, 3.0, 333)
    s = (r * r).astype(np.float32)
    x = (s.astype(np.float64) - float(sur.norm[0])) * float(sur.norm[1])
    y_ref, _ = mlp_ref.forward(p, x)
    y_gpu = sur.network(s, accurate=True)
    # split-bf16 activations keep ~16 bits: outputs agree to ~1e-4 of their scale
    assert np.max(np.abs(y_gpu - y_ref)) <= 2e-3 * max(1.0, np.max(np.abs(y_ref)))
    t = rng.normal(0, 1, (s.size, 2)).astype(np.float32)
    loss_gpu, g_gpu = sur.gradients(s, t, wf=0.7, accurate=True)
    loss_ref, g_ref = mlp_ref.loss_and_grad(p, x, t.astype(np.float64), wf=0.7)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * loss_ref
    # the backward GEMMs take bf16 operands: compare the gradient as a vector
    rel = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    cos = float(np.dot(g_gpu, g_ref) / (np.linalg.norm(g_gpu) * np.linalg.norm(g_ref)))
    print(f"gradient relative L2 error {rel:.2e}, cosine {cos:.6f}")
    assert rel <= 2e-2 and cos >= 0.9995
    for name, sl in (("w1", slice(0, 64)), ("W2", slice(128, 4224)), ("W3", slice(4288, 4416))):
        part = np.linalg.norm(g_gpu[sl] - g_ref[sl]) / np.linalg.norm(g_ref[sl])
        assert part <= 3e-2, name


def test_training_reaches_accuracy(surrogate):
    err = surrogate.errors()
    print("surrogate accuracy vs float64 codegen:", err, "final loss", float(surrogate.losses[-1]))
    assert surrogate.losses[-1] < surrogate.losses[0] * 1e-3
    assert err["fr_rel_rms"] < 1e-2
    assert err["fr_rel_rms_of_total"] < 1e-4


def _jittered_fcc(cells, seed=0, density=0.8, jitter=0.05):
    """fcc at density 0.8 with N(0, 0.05) jitter, the costly potential
    (r_cut 3, list skin 0.3): the state the benchmark measures the force
    error on (there with 64^3 cells)."""
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC, generate_positions

    pos = generate_positions(FCC, cells, (1.0, 1.0, 1.0))
    box = np.array(cells, dtype=np.float64)
    scale = (pos.shape[0] / np.prod(box) / density) ** (1 / 3)
    box, pos = box * scale, pos * scale
    rng = np.random.default_rng(seed)
    pos = pos + rng.normal(0.0, jitter, size=pos.shape)
    img = np.floor(pos / box)
    n = pos.shape[0]
    sim = Simulation()
    sim.box_vectors = box
    sim.positions = pos - img * box
    sim.velocities = np.zeros_like(pos)
    sim.betas = np.zeros_like(pos)
    sim.image_positions = img.astype(np.int32)
    sim.masses = np.ones((n, 1))
    sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    sim.set_pair_potential(expensive_string(), 3.0)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=256, method_str="cell list")
    return sim


def test_surrogate_force_error_target_on_lattice(surrogate):
    """The force RMS error of the surrogate against the float64 generated
    code stays within the 1e-4 target on the jittered fcc lattice (32^3
    cells, 131,072 particles)."""
    sim = _jittered_fcc((32, 32, 32))
    f64 = sim.get_forces()
    sim.set_pair_surrogate(surrogate)
    fnn = sim.get_forces()
    err = float(np.sqrt(np.mean((fnn - f64) ** 2) / np.mean(f64 ** 2)))
    print(f"surrogate force relative RMS error on the jittered lattice: {err:.2e}")
    assert err <= 1e-4


def _liquid(seed=0, cells=(10, 10, 10)):
    from dompap_gb300 import Simulation
    from dompap_gb300.positions import FCC

    np.random.seed(seed)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=FCC, cells=cells, lattice_constants=(1, 1, 1))
    sim.set_masses(masses=1.0)
    sim.set_density(density=0.8)
    sim.set_random_velocities(temperature=1.5)
    sim.set_pair_potential(expensive_string(), 3.0)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=256, method_str="cell list")
    sim.set_integrator(time_step=0.004, target_temperature=1.5, temperature_damping_time=0.1)
    sim.run(400)  # melt
    return sim


def test_surrogate_forces_and_energy(surrogate):
    sim = _liquid()
    f64 = sim.get_forces()
    u64 = sim.get_potential_energy()
    w64 = sim.get_virial()
    sim.set_pair_surrogate(surrogate)
    fnn = sim.get_forces()
    unn = sim.get_potential_energy()
    wnn = sim.get_virial()
    err = np.sqrt(np.mean((fnn - f64) ** 2) / np.mean(f64 ** 2))
    n = sim.number_of_particles()
    print(f"surrogate force relative RMS error {err:.2e}; U/N {unn / n:.6f} vs {u64 / n:.6f}; "
          f"W/N {wnn / n:.5f} vs {w64 / n:.5f}")
    assert err < 1e-3
    assert abs(unn - u64) <= 1e-3 * abs(u64)
    assert abs(wnn - w64) <= 2e-3 * abs(w64)
    sim.set_pair_surrogate(None)
    assert np.array_equal(sim.get_forces(), f64)


def test_surrogate_forces_deterministic_and_balanced(surrogate):
    """Each unique pair is evaluated once and its force added to both
    particles through 64-bit fixed-point sums: repeated evaluations are
    bit-identical, and the total force vanishes up to the float32 rounding of
    each particle's own sum (a pair added to one side only would leave a
    total of the order of the force magnitudes)."""
    sim = _liquid(seed=2)
    sim.set_pair_surrogate(surrogate)
    f1 = sim.get_forces()
    f2 = sim.get_forces()
    assert np.array_equal(f1, f2)
    assert np.max(np.abs(f1.sum(axis=0))) <= 1e-5 * np.sum(np.abs(f1))
    assert np.max(np.abs(f1)) > 1.0


def test_surrogate_mode_half_lists_export_full(surrogate):
    """The surrogate mode keeps neighbour lists of partners j > i only (its
    kernels use each pair once); the export closes them into the reference's
    full list at the list's reference positions, without a rebuild, and forces
    do not change across the export."""
    from oracle import numpy_ref as ref

    sim = _liquid(seed=4)
    sim.set_pair_surrogate(surrogate)
    f1 = sim.get_forces()
    updates = sim.number_of_neighbor_list_updates
    exported = np.array(sim.neighbor_list)
    assert sim.number_of_neighbor_list_updates == updates
    want, _ = ref.neighbor_list_double_loop(np.array(sim.positions_neighbour_list), np.array(sim.box_vectors),
                                            3.0 + 0.3, exported.shape[1])
    assert np.array_equal(exported, want)
    f2 = sim.get_forces()
    assert np.array_equal(f1, f2)


def test_tcgen05_pass_matches_mma_sync_pass(surrogate, monkeypatch):
    """The surrogate's 128 x 64 x 64 layer on the fifth-generation tensor
    cores (tcgen05.mma, TMEM accumulator) and on mma.sync give the same
    forces, energy and virial: the same bf16 operands and fp32 accumulation,
    summed in another order."""
    out = {}
    for tag, env in (("tc", "tcgen05"), ("mma", "mma")):
        monkeypatch.setenv("DOMPAP_MLP_TENSOR", env)
        sim = _liquid(seed=3)
        sim.set_pair_surrogate(surrogate)
        out[tag] = (sim.get_forces(), sim.get_potential_energy(), sim.get_virial())
    f_tc, u_tc, w_tc = out["tc"]
    f_mm, u_mm, w_mm = out["mma"]
    err = np.sqrt(np.mean((f_tc - f_mm) ** 2) / np.mean(f_mm ** 2))
    print(f"tcgen05 vs mma.sync: force relative RMS {err:.2e}, U {u_tc:.9f} vs {u_mm:.9f}, W {w_tc:.9f} vs {w_mm:.9f}")
    assert err <= 1e-5
    assert abs(u_tc - u_mm) <= 1e-6 * abs(u_mm)
    assert abs(w_tc - w_mm) <= 1e-6 * abs(w_mm)


def test_surrogate_nve_drift_and_speed(surrogate):
    from dompap_gb300 import _lib

    sim = _liquid(seed=1)
    sim.set_integrator(time_step=0.002)

    def etot():
        return sim.get_potential_energy() + sim.get_kinetic_energy()

    def drift(steps=1000, blocks=5):
        e = [etot()]
        for _ in range(blocks):
            sim.run_leap_frog(steps // blocks)
            e.append(etot())
        return (e[-1] - e[0]) / sim.number_of_particles(), np.std(e) / sim.number_of_particles()

    d64 = drift()
    ms64 = _lib.ctypes.c_float(0.0)
    _lib.check(_lib.load().dp_time_kernel(sim._h, _lib.DP_KERNEL_FORCES, 20, _lib.ctypes.byref(ms64)))
    sim.set_pair_surrogate(surrogate)
    dnn = drift()
    msnn = _lib.ctypes.c_float(0.0)
    _lib.check(_lib.load().dp_time_kernel(sim._h, _lib.DP_KERNEL_FORCES, 20, _lib.ctypes.byref(msnn)))
    print(f"NVE energy change per particle over 1000 steps: fp64 codegen {d64[0]:+.2e} (std {d64[1]:.1e}), "
          f"surrogate {dnn[0]:+.2e} (std {dnn[1]:.1e}); force kernel {ms64.value:.3f} ms vs "
          f"{msnn.value:.3f} ms")
    assert abs(dnn[0]) < 5e-3
    assert msnn.value < ms64.value


def test_surrogate_ensemble_matches_float64_code(surrogate):
    """Langevin ensemble averages (T, U/N, P) of the 4,000-particle liquid with
    the surrogate agree with those of the float64 generated code within 4
    combined standard errors (block averages of independent runs)."""

    def ensemble(use_surrogate):
        sim = _liquid(seed=6)
        if use_surrogate:
            sim.set_pair_surrogate(surrogate)
        n = sim.number_of_particles()
        sim.run(400)
        obs = {"T": [], "U": [], "P": []}
        for _ in range(100):
            sim.run(20)
            obs["T"].append(sim.get_temperature())
            obs["U"].append(sim.get_potential_energy() / n)
            obs["P"].append(sim.get_pressure())
        return obs

    a, b = ensemble(False), ensemble(True)
    for key in ("T", "U", "P"):
        ma = np.array([x.mean() for x in np.array_split(np.array(a[key]), 10)])
        mb = np.array([x.mean() for x in np.array_split(np.array(b[key]), 10)])
        err = np.hypot(ma.std(ddof=1), mb.std(ddof=1)) / np.sqrt(10)
        print(f"{key}: float64 code {ma.mean():.4f}  surrogate {mb.mean():.4f}  (+- {err:.4f})")
        assert abs(ma.mean() - mb.mean()) < 4 * err + 1e-3 * abs(ma.mean()), key
