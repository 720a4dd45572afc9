"""Pin the oracle: ``oracle.numpy_ref`` against golden vectors produced by the
unmodified reference (tests/golden/make_golden.py) and the reference's own
test values. CPU only.

Pair sets, wrap, images and the integrator arithmetic must match bit for bit.
Values that go through ``pow`` (the pair potential) may differ in the last
bits, because NumPy's vectorised ``pow`` over an array and its scalar ``pow``
(which the fixtures used, element by element) are different routines; those
are compared at 1e-13 relative to the quantity's scale.
"""
import numpy as np
import pytest

from conftest import CONFIG_TAGS, config_of
from oracle import numpy_ref as ref

RTOL = 1e-13


def close(got, want, scale=None):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    scale = np.max(np.abs(want)) if scale is None else scale
    assert got.shape == want.shape
    err = np.max(np.abs(got - want)) if got.size else 0.0
    assert err <= RTOL * max(scale, 1e-300), (err, scale)


def _pot(cfg, tag):
    if tag == "hard3d":
        u, f, c, _ = ref.harmonic_repulsive()
        return u, f, c
    return ref.make_pair_potential(str(cfg["pot"]), float(cfg["r_cut"]))


def _params(cfg):
    n = cfg["positions"].shape[0]
    if "types" in cfg:
        t = cfg["types"]
        return cfg["sigma_table"][t[:, None], t[None, :]], cfg["epsilon_table"][t[:, None], t[None, :]]
    sig = cfg.get("sigma_table", np.float64(1.0))
    eps = cfg.get("epsilon_table", np.float64(1.0))
    sig = float(sig) if np.ndim(sig) == 0 else sig
    eps = float(eps) if np.ndim(eps) == 0 else eps
    assert np.ndim(sig) in (0, 2) and (np.ndim(sig) == 0 or sig.shape == (n, n))
    return sig, eps


# ---------------------------------------------------------------- unit vectors
def test_neighbor_lists_reference_tests(golden_unit):
    # tests/test_neighbor_list.py:12-51 inputs and expected arrays
    nl, _ = ref.neighbor_list_double_loop(golden_unit["nl3d/positions"], np.array([6.0] * 3), 1.5, 4)
    assert np.array_equal(nl, golden_unit["nl3d/nlist"])
    assert np.array_equal(nl, np.array([[1, 2, 3, 5], [0, 2, 3, -1], [0, 1, 3, -1], [0, 1, 2, -1],
                                        [-1, -1, -1, -1], [0, -1, -1, -1]]))
    nl, _ = ref.neighbor_list_double_loop(golden_unit["nl2d/positions"], np.array([6.0] * 2), 1.5, 4)
    assert np.array_equal(nl, golden_unit["nl2d/nlist"])


def test_skin_trigger(golden_unit):
    pos = np.array([[0, 0, 0], [1, 1, 1]], dtype=np.float64)
    old = np.array([[0.5, 0, 0], [1, 1, 1]], dtype=np.float64)
    got = [ref.neighbor_list_is_old(pos, old, np.array([5.0] * 3), s) for s in golden_unit["skin/skins"]]
    assert got == list(golden_unit["skin/is_old"])
    # tests/test_neighbor_list.py:94-104: +-0.01 around skin/2, and the periodic image
    skin = 0.5
    p = np.zeros((2, 3))
    o = np.zeros((2, 3))
    assert not ref.neighbor_list_is_old(p, o, np.array([5.0] * 3), skin)
    o[0] = [skin / 2 - 0.01, 0, 0]
    assert not ref.neighbor_list_is_old(p, o, np.array([5.0] * 3), skin)
    o[0] = [skin / 2 + 0.01, 0, 0]
    assert ref.neighbor_list_is_old(p, o, np.array([5.0] * 3), skin)
    o[0] = [5.0, 0, 0]
    assert not ref.neighbor_list_is_old(p, o, np.array([5.0] * 3), skin)


@pytest.mark.parametrize("tag,expr,rc", [("harm", "(1-r)**2", 1.0), ("lj", "4*(r**-12-r**-6)", 2.5),
                                         ("ljinf", "4*(r**-12-r**-6)", np.inf), ("exp", None, 3.0)])
def test_pair_potential_values(golden_unit, tag, expr, rc):
    if expr is None:
        expr = str(golden_unit["pot_exp/expr"])
    u, f, c = ref.make_pair_potential(expr, rc)
    r = golden_unit[f"pot_{tag}/r"]
    for name, fn in (("u", u), ("f", f), ("c", c)):
        want = golden_unit[f"pot_{tag}/{name}"]
        got = fn(r)
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=RTOL * np.max(np.abs(want)))


def test_pair_potential_reference_scalars():
    # tests/test_potential.py:20-39
    u, f, c = ref.make_pair_potential("(1-r)**2", 1.0)
    assert u(0.5) == 0.25 and f(0.5) == 1.0 and c(0.5) == 2.0
    u, f, c = ref.make_pair_potential("4*(r**-12-r**-6)", np.inf)
    rmin = 2 ** (1 / 6)
    assert np.isclose(u(rmin), -1.0, atol=1e-6)
    assert np.isclose(f(1.0), 24.0, atol=1e-6)
    assert np.isclose(c(1.0), 456.0, atol=1e-6)
    assert np.isclose(c(rmin), 57.14643787, atol=1e-6)


def test_hardcoded_potential(golden_unit):
    u, f, c, rc = ref.harmonic_repulsive()
    r = golden_unit["pot_hard/r"]
    assert np.array_equal(u(r), golden_unit["pot_hard/u"])
    assert np.array_equal(f(r), golden_unit["pot_hard/f"])
    assert rc == 1.0


def test_wrap_into_box(golden_unit):
    p = golden_unit["wrap/in"].copy()
    img = np.zeros(p.shape, dtype=np.int32)
    ref.wrap_into_box(p, img, np.array([2.0] * 3))
    assert np.array_equal(p, golden_unit["wrap/positions"])
    assert np.array_equal(img, golden_unit["wrap/images"])


def test_gjf_and_leapfrog_steps(golden_unit):
    g = {k.split("/", 1)[1]: v for k, v in golden_unit.items() if k.startswith("gjf/")}
    pos, vel, beta = ref.gjf_step(g["positions"], g["velocities"], g["betas"], g["forces"], g["masses"], 0.005, 1.3,
                                  0.1, g["normals"])
    assert np.array_equal(pos, g["new_positions"])
    assert np.array_equal(vel, g["new_velocities"])
    assert np.array_equal(beta, g["new_betas"])
    pos, vel = ref.leapfrog_step(g["positions"], g["velocities"], g["forces"], g["masses"], 0.005)
    assert np.array_equal(pos, golden_unit["leapfrog/new_positions"])
    assert np.array_equal(vel, golden_unit["leapfrog/new_velocities"])


def test_sigma2_epsilon4_semantics(golden_unit):
    # tests/test_potential.py:81-140: U = 1, F = -+4 (no 1/sigma chain-rule factor)
    pos = np.array([[0, 0, 0], [1, 0, 0]], dtype=np.float64)
    box = np.array([3.0] * 3)
    u, f, c = ref.make_pair_potential("(1-r)**2", 1.0)
    nl = np.array([[1], [0]], dtype=np.int32)
    assert ref.energy_neighbor_list(pos, box, u, nl, 2.0, 4.0) == 1.0 == golden_unit["sig2eps4/energy"]
    forces = ref.forces_neighbor_list(pos, box, f, nl, 2.0, 4.0)
    assert np.array_equal(forces, golden_unit["sig2eps4/forces"])
    assert np.allclose(forces, [[-4, 0, 0], [4, 0, 0]])


def test_doctest_values(golden_unit):
    # Simulation.py:553-555: default system scaled by 0.5 -> U = 167.06442443573454
    pos = ref.generate_positions([[0, 0, 0]], (5, 5, 5), (1, 1, 1)) * 0.5
    box = np.array([2.5] * 3)
    u, f, c = ref.make_pair_potential("(1-r)**2", 1.0)
    nl, _ = ref.neighbor_list_double_loop(pos, box, 1.0 + 1.0, 512)
    e = ref.energy_neighbor_list(pos, box, u, nl)
    assert e == golden_unit["doctest/energy_scaled"] == 167.06442443573454
    # :602-605: particle 0 shifted to x = 0.5 -> F_x = -1
    pos = ref.generate_positions([[0, 0, 0]], (5, 5, 5), (1, 1, 1))
    pos[0] = [0.5, 0, 0]
    box = np.array([5.0] * 3)
    nl, _ = ref.neighbor_list_double_loop(ref.generate_positions([[0, 0, 0]], (5, 5, 5), (1, 1, 1)), box, 2.0, 512)
    forces = ref.forces_neighbor_list(pos, box, f, nl)
    assert np.array_equal(forces[0], golden_unit["doctest/force0"])
    # :1213-1215: Laplacian of particle 0 = 12
    pos = ref.generate_positions([[0, 0, 0]], (5, 5, 5), (1, 1, 1))
    nl, _ = ref.neighbor_list_double_loop(pos, box, 2.0, 512)
    lap = ref.laplacian_neighbor_list(pos, box, f, c, nl)
    assert lap[0] == golden_unit["doctest/laplacian0"] == 12.0


# ------------------------------------------------------------- configurations
@pytest.mark.parametrize("tag", CONFIG_TAGS)
def test_configuration(golden_configs, tag):
    cfg = config_of(golden_configs, tag)
    pos, box = cfg["positions"], cfg["box"]
    u, f, c = _pot(cfg, tag)
    sig, eps = _params(cfg)
    smax = float(np.max(ref.pair_matrix(sig, pos.shape[0])))
    cutoff = smax * float(cfg["r_cut"]) + float(cfg["skin"])
    k = cfg["nlist"].shape[1]
    nl, counts = ref.neighbor_list_double_loop(pos, box, cutoff, k)
    assert np.array_equal(nl, cfg["nlist"]), "pair set / order differs from the reference"
    assert counts.max() <= k
    forces = ref.forces_neighbor_list(pos, box, f, nl, sig, eps)
    close(forces, cfg["forces"])
    if "energy" in cfg:
        e = ref.energy_neighbor_list(pos, box, u, nl, sig, eps)
        close(e, cfg["energy"], ref.pair_terms_abs_sum(pos, box, u, nl, sig, eps))
    w, w_abs = ref.virial_double_loop(pos, box, f, sig, eps, return_abs=True)
    close(w, cfg["virial"], w_abs)
    lap = ref.laplacian_neighbor_list(pos, box, f, c, nl, sig, eps)
    close(lap, cfg["laplacian"])
    if "rdf_g" in cfg:
        r, g = ref.radial_distribution_function(pos, pos, box, cfg["rdf_bins"])
        assert np.array_equal(r, cfg["rdf_r"]) and np.array_equal(g, cfg["rdf_g"])


def test_nve_trajectory(golden_traj):
    t = {k.split("/", 1)[1]: v for k, v in golden_traj.items() if k.startswith("nve/")}
    sys_ = ref.OracleSystem(t["positions0"], t["velocities0"], np.ones(t["positions0"].shape[0]), t["box"],
                            "4*(r**-12-r**-6)", 2.5, 0.3)
    sys_.images = t["images0"].copy()
    sys_.dt = 0.005
    for _ in range(int(t["steps"])):
        sys_.step_leap_frog()
    close(sys_.positions, t["positions"], 1.0)
    close(sys_.velocities, t["velocities"], 1.0)
    assert np.array_equal(sys_.images, t["images"])


def test_gjf_tau_inf_trajectory(golden_traj):
    t = {k.split("/", 1)[1]: v for k, v in golden_traj.items() if k.startswith("gjfinf/")}
    sys_ = ref.OracleSystem(t["positions0"], t["velocities0"], np.ones(t["positions0"].shape[0]), t["box"],
                            "(1-r)**2", 1.0, 0.2)
    sys_.images = t["images0"].copy()
    sys_.dt, sys_.temperature, sys_.damping_time = 0.01, 0.5, np.inf
    rng = np.random.default_rng(0)
    for _ in range(int(t["steps"])):
        sys_.step_gjf(rng.normal(size=sys_.positions.shape))
    close(sys_.positions, t["positions"], 1.0)
    close(sys_.velocities, t["velocities"], 1.0)
    assert np.array_equal(sys_.images, t["images"])


def test_rdf_per_type_pair():
    """g(r) of each type pair of the binary configuration: the oracle on the
    type subsets equals the reference's own get_radial_distribution_function
    (dompap/positions.py:58-87) called on the same subsets."""
    from conftest import load_golden

    gold = load_golden("golden_rdf_types.npz")
    cfg = load_golden("golden_configs.npz")
    pos, box = cfg["wahn/positions"], cfg["wahn/box"]
    types = cfg["wahn/types"].reshape(-1)
    for a, b, key in ((0, 0, "AA"), (0, 1, "AB"), (1, 1, "BB")):
        r, g = ref.radial_distribution_function(pos[types == a], pos[types == b], box, gold["bins"])
        assert np.array_equal(r, gold[f"{key}/r"])
        np.testing.assert_allclose(g, gold[f"{key}/g"], rtol=1e-13, atol=0)


def test_double_loop_methods():
    """The oracle's double-loop force and energy methods against the
    reference's own (dompap/potential.py:103-160,191-250,298-324), including
    the asymmetric epsilon(n, m) where "double loop single core" (Newton's
    third law with (n, m), n < m) and the upper-triangle energies differ from
    the neighbour-list sums."""
    from conftest import config_of, load_golden

    gold = load_golden("golden_methods.npz")
    cfgs = load_golden("golden_configs.npz")
    for tag in ("callable", "wahn", "harm2d"):
        c = config_of(cfgs, tag)
        pos, box = c["positions"], c["box"]
        u, f, _ = ref.make_pair_potential(str(c["pot"]), float(c["r_cut"]))
        if "types" in c:
            t = c["types"].reshape(-1)
            sig, eps = c["sigma_table"][t[:, None], t[None, :]], c["epsilon_table"][t[:, None], t[None, :]]
        elif "sigma_table" in c:
            sig, eps = c["sigma_table"], c["epsilon_table"]
        else:
            sig, eps = 1.0, 1.0
        for method, fn in (("double loop", ref.forces_double_loop),
                           ("double loop single core", ref.forces_double_loop_single_core)):
            want = gold[f"{tag}/forces/{method}"]
            got = fn(pos, box, f, sig, eps)
            assert np.sqrt(np.mean((got - want) ** 2) / np.mean(want ** 2)) <= 1e-13, (tag, method)
        e = ref.energy_double_loop(pos, box, u, sig, eps)
        assert abs(e - gold[f"{tag}/energy/double loop"]) <= 1e-12 * abs(gold[f"{tag}/energy/double loop"]), tag
