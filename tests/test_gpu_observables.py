"""GPU parity of the neighbour-list skin trigger, the per-type g(r) and the
binary-mixture (Wahnstrom-type) Langevin ensemble.

* Skin trigger, ``neighbor_list_is_old`` (dompap/neighbor_list.py:183-201), on
  the reference's own cases (tests/test_neighbor_list.py:94-118): a particle
  skin/2 -+ 0.01 from where the list was built, one that moved to its own
  periodic image, and twenty skins around a displacement of 0.5. Both device
  tests decide exactly as the reference, bit for bit: ``k_skin_check`` (what
  ``update_neighbor_list(check=True)`` and the start of ``run`` launch) and the
  test inside the step kernels (fused ``dp_step`` and the separate
  ``k_integrate``), read back as whether the next step rebuilt the list.
* g(r) of each type pair (dompap/positions.py:58-87 on the type subsets),
  against the reference's own output at 1e-12.
* Binary LJ mixture (sigma AA/AB/BB = 1.0/1.1/1.2, masses 2:1, r_cut 2.5 sigma,
  T = 0.7): T, U/N, P and the per-type g(r) from the GPU run and from the
  oracle's own Langevin run agree within 4 (5 for g(r)) combined standard
  errors of their block averages.
"""
import ctypes

import numpy as np
import pytest

from conftest import config_of, load_golden
from gpu_helpers import sim_from_config
from oracle import numpy_ref as ref

pytestmark = pytest.mark.gpu


def _lib():
    from dompap_gb300 import _lib

    return _lib


def _system(reference_positions, skin, box=5.0):
    """Particles with their list built at ``reference_positions`` (box 5^3,
    (1-r)^2 with r_cut 1, zero velocities and forces beyond r_cut)."""
    from dompap_gb300 import Simulation

    p = np.array(reference_positions, dtype=np.float64)
    n = p.shape[0]
    sim = Simulation()
    sim.box_vectors = np.full(3, float(box))
    sim.positions = p
    sim.velocities = np.zeros((n, 3))
    sim.betas = np.zeros((n, 3))
    sim.image_positions = np.zeros((n, 3), dtype=np.int32)
    sim.masses = np.ones((n, 1))
    sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_neighbor_list(skin=float(skin), max_number_of_neighbors=8)
    sim.update_neighbor_list(check=False)
    assert np.array_equal(sim.positions_neighbour_list, p)
    return sim


def _device_is_old(sim, positions):
    """update_neighbor_list(check=True) on the device: did it rebuild?"""
    lib = _lib()
    sim.positions = np.array(positions, dtype=np.float64)
    sim._push()
    rebuilt = ctypes.c_int(-1)
    lib.check(lib.load().dp_update_neighbor_list(sim._h, 1, ctypes.byref(rebuilt)))
    assert rebuilt.value in (0, 1)
    return bool(rebuilt.value)


def _reference_cases(golden_unit):
    """(list positions, current positions, skin, reference is_old)."""
    cases = []
    cur = [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]
    skin = 0.5
    # tests/test_neighbor_list.py:95-104
    cases.append(([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]], cur, skin, False))
    cases.append(([[skin / 2 - 0.01, 0.0, 0.0], [0.0, 0.0, 0.0]], cur, skin, False))
    cases.append(([[skin / 2 + 0.01, 0.0, 0.0], [0.0, 0.0, 0.0]], cur, skin, True))
    cases.append(([[0.0 + 5.0, 0.0, 0.0], [0.0, 0.0, 0.0]], cur, skin, False))
    # tests/test_neighbor_list.py:107-118: the reference's decisions for 20 skins
    for s, old in zip(golden_unit["skin/skins"], golden_unit["skin/is_old"]):
        cases.append(([[0.5, 0.0, 0.0], [1.0, 1.0, 1.0]], [[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]], float(s), bool(old)))
    return cases


def test_skin_check_kernel_reference_cases(golden_unit):
    cases = _reference_cases(golden_unit)
    for built_at, now, skin, want in cases:
        # the oracle and the reference agree on every case (pinned on the CPU too)
        assert ref.neighbor_list_is_old(np.array(now, float), np.array(built_at, float), np.full(3, 5.0),
                                        skin) == want
        sim = _system(built_at, skin)
        got = _device_is_old(sim, now)
        assert got == want, (built_at, now, skin)
        # a rebuild makes the current positions the list's reference positions
        expect_ref = np.array(now if want else built_at, dtype=np.float64)
        assert np.array_equal(sim.positions_neighbour_list, expect_ref)


@pytest.mark.parametrize("fused", ["1", "0"])
def test_step_skin_test_reference_cases(golden_unit, monkeypatch, fused):
    """The skin test at the end of each step (dp_step, or k_integrate when the
    step is not fused): particle 0 starts where the list was built and moves by
    the reference's displacement in one NVE step (zero forces: the particles
    are more than r_cut apart); the second step of the run rebuilds the list
    exactly when the reference calls the list old."""
    monkeypatch.setenv("DOMPAP_FUSED_STEP", fused)
    dt = 0.01
    checked = 0
    for s, want in zip(golden_unit["skin/skins"], golden_unit["skin/is_old"]):
        start = [[0.5, 0.0, 0.0], [1.0, 1.0, 1.0]]
        sim = _system(start, float(s))
        sim.set_integrator(time_step=dt)
        v = np.zeros((2, 3))
        v[0, 0] = -0.5 / dt  # x: 0.5 -> 0.0 after one step
        sim.velocities = v
        r0 = sim._stats().rebuilds
        sim.run_leap_frog(2)
        rebuilt = sim._stats().rebuilds - r0
        assert rebuilt == int(bool(want)), (s, want)
        checked += 1
    assert checked == 20


def test_rdf_per_type_pair_matches_reference(golden_configs):
    gold = load_golden("golden_rdf_types.npz")
    cfg = config_of(golden_configs, "wahn")
    sim = sim_from_config(cfg, "wahn", method="cell list")
    for a, b, key in ((0, 0, "AA"), (0, 1, "AB"), (1, 1, "BB")):
        r, g = sim.get_radial_distribution_function(gold["bins"], type_a=a, type_b=b)
        assert np.array_equal(r, gold[f"{key}/r"]), key
        np.testing.assert_allclose(g, gold[f"{key}/g"], rtol=1e-12, atol=0, err_msg=key)
    # the untyped g(r) is the particle-number weighted sum of the type pairs
    r, g_all = sim.get_radial_distribution_function(gold["bins"])
    t = cfg["types"].reshape(-1)
    na, nb = int(np.sum(t == 0)), int(np.sum(t == 1))
    n = na + nb
    mix = (na * na * gold["AA/g"] + 2 * na * nb * gold["AB/g"] + nb * nb * gold["BB/g"]) / (n * n)
    np.testing.assert_allclose(g_all, mix, rtol=1e-12, atol=1e-12)


def _block_mean(x, nblocks=10):
    x = np.asarray(x)
    m = np.array([v.mean(axis=0) for v in np.array_split(x, nblocks)])
    return m.mean(axis=0), m.std(axis=0, ddof=1) / np.sqrt(nblocks)


@pytest.mark.slow
def test_binary_mixture_ensemble_matches_oracle():
    """Wahnstrom-type mixture, 1,000 particles (simple cubic 10^3, density 0.75,
    seeded 50:50 types, masses A:B = 2:1), LJ with r_cut 2.5 sigma and the
    reference's force ``eps f(r/sigma) d/r``, skin 0.5, G-JF T = 0.7,
    dt = 0.004, damping time 0.2. The GPU equilibrates the liquid from the
    lattice (20,000 steps: at T = 0.7 the A-A structure relaxes slowly), then
    the GPU and the oracle each sample 1,200 steps from that state with their
    own noise: the same ensemble."""
    from dompap_gb300 import Simulation

    rng = np.random.default_rng(31)
    np.random.seed(31)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0.0, 0.0, 0.0],), cells=(10, 10, 10), lattice_constants=(1, 1, 1))
    n = sim.number_of_particles()
    types = np.zeros(n, dtype=np.int32)
    types[rng.permutation(n)[: n // 2]] = 1
    masses = np.where(types == 0, 2.0, 1.0)
    sig_t = np.array([[1.0, 1.1], [1.1, 1.2]])
    sim.set_types([int(t) for t in types])
    sim.set_masses(masses=list(masses))
    sim.set_density(density=0.75)
    sim.set_random_velocities(temperature=0.7)
    sim.set_pair_potential("4*(r**-12-r**-6)", 2.5)
    sim.set_pair_potential_parameters(sigma=lambda a, b: sig_t[types[a], types[b]], epsilon=1.0)
    sim.set_neighbor_list(skin=0.5, max_number_of_neighbors=256, method_str="cell list")
    sim.set_integrator(time_step=0.004, target_temperature=0.7, temperature_damping_time=0.2)
    box = np.array(sim.box_vectors)
    sim.run(20000)
    pos0, vel0 = np.array(sim.positions), np.array(sim.velocities)
    samples, stride = 120, 10
    r_bins = np.linspace(0.7, 0.5 * float(box[0]), 46)
    pairs = ((0, 0, "AA"), (0, 1, "AB"), (1, 1, "BB"))
    vol = float(np.prod(box))

    g = {"T": [], "U": [], "P": []}
    g.update({k: [] for _, _, k in pairs})
    for _ in range(samples):
        sim.run(stride)
        g["T"].append(sim.get_temperature())
        g["U"].append(sim.get_potential_energy() / n)
        g["P"].append(sim.get_pressure())
        for a, b, k in pairs:
            g[k].append(sim.get_radial_distribution_function(r_bins, type_a=a, type_b=b)[1])

    sig = sig_t[types[:, None], types[None, :]]
    o = ref.OracleSystem(pos0, vel0, masses, box, "4*(r**-12-r**-6)", 2.5, 0.5, sigma=sig, epsilon=1.0,
                         max_neighbors=256)
    o.dt, o.temperature, o.damping_time = 0.004, 0.7, 0.2
    h = {k: [] for k in g}
    m = masses[:, None]
    for _ in range(samples):
        for _ in range(stride):
            o.step_gjf(rng.normal(size=(n, 3)))
        o.update_neighbor_list()
        mv2 = float(np.sum(m * o.velocities ** 2))
        h["T"].append(mv2 / (3 * n))
        h["U"].append(ref.energy_neighbor_list(o.positions, box, o.u, o.nlist, sig, 1.0) / n)
        w = ref.virial_double_loop(o.positions, box, o.f, sig, 1.0)
        h["P"].append(w / vol + mv2 / 3 / vol)
        for a, b, k in pairs:
            h[k].append(ref.radial_distribution_function(o.positions[types == a], o.positions[types == b], box,
                                                         r_bins)[1])
    for key in ("T", "U", "P"):
        mg, eg = _block_mean(g[key])
        mo, eo = _block_mean(h[key])
        print(f"{key}: GPU {mg:.4f} +- {eg:.4f}   oracle {mo:.4f} +- {eo:.4f}")
        assert abs(mg - mo) < 4 * np.hypot(eg, eo) + 1e-3 * abs(mo), key
    for _, _, key in pairs:
        mg, eg = _block_mean(g[key])
        mo, eo = _block_mean(h[key])
        z = np.abs(mg - mo) / (np.hypot(eg, eo) + 2e-3)
        pg, po = int(np.argmax(mg)), int(np.argmax(mo))
        print(f"g_{key}(r): first peak GPU {mg[pg]:.3f} at bin {pg}, oracle {mo[po]:.3f} at bin {po}; "
              f"largest deviation {z.max():.2f} standard errors")
        assert abs(pg - po) <= 1 and mg[pg] > 1.5, key
        assert z.max() < 5.0, key
