"""Generate the golden fixtures in this folder by running the UNMODIFIED dompap
reference (pure-Python mode: ``oracle/stubs`` supplies a pass-through ``numba``,
a ``toml`` shim and a no-op ``matplotlib``).

Run in a checkout that has the reference source next to it::

    python tests/golden/make_golden.py --reference PATH   (or DOMPAP_REFERENCE=PATH)

It writes ``golden_*.npz``, ``checkpoint_ref.csv/.toml`` and ``lammps_ref.*``. Every array is produced by calling the reference's
own functions / ``Simulation`` methods on seeded inputs; nothing here restates
the reference's arithmetic. The fixtures are what ``tests/`` pin the oracle and
the CUDA path against, on machines where the reference is absent.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

FCC = ((0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5))
LJ = "4*(r**-12-r**-6)"
EXPENSIVE_RAW = "4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r)"


def shifted_force_string(expr: str, r_cut: float) -> str:
    """``u(r) - u(rc) - (r - rc) u'(rc)`` as a SymPy string with 17-digit
    constants (the smooth shift goes into the expression; dompap itself only
    shifts the value)."""
    import sympy as sp

    r = sp.symbols("r")
    u = sp.sympify(expr)
    u_rc = sp.N(u.subs(r, r_cut), 30)
    du_rc = sp.N(sp.diff(u, r).subs(r, r_cut), 30)
    return f"{expr} - ({float(u_rc)!r}) - (r - {float(r_cut)!r})*({float(du_rc)!r})"


EXPENSIVE = shifted_force_string(EXPENSIVE_RAW, 3.0)


def import_reference(path: str):
    sys.path.insert(0, path)
    sys.path.insert(0, os.path.join(REPO, "oracle", "stubs"))
    import dompap  # noqa: F401

    return dompap


def build_sim(Simulation, unit_cell, cells, density, pot, r_cut, skin, rng, jitter, kmax=256):
    """A reference ``Simulation`` on a jittered lattice, via its public setters."""
    sim = Simulation()
    dim = len(unit_cell[0])
    sim.set_positions(unit_cell_coordinates=unit_cell, cells=cells, lattice_constants=(1.0,) * dim)
    sim.set_masses(masses=1.0)
    sim.set_density(density=density)
    sim.positions = sim.positions + rng.normal(0.0, jitter, size=sim.positions.shape)
    sim.wrap_into_box()
    sim.velocities = rng.normal(0.0, 1.0, size=sim.positions.shape)
    sim.set_pair_potential(pair_potential_str=pot, r_cut=r_cut)
    sim.set_neighbor_list(skin=skin, max_number_of_neighbors=kmax)
    return sim


def record_sim(out: dict, tag: str, sim, sigma=None, epsilon=None, types=None, rdf_bins=None):
    t0 = time.time()
    out[f"{tag}/positions"] = sim.positions.copy()
    out[f"{tag}/velocities"] = sim.velocities.copy()
    out[f"{tag}/masses"] = sim.masses.copy()
    out[f"{tag}/box"] = sim.box_vectors.copy()
    out[f"{tag}/pot"] = np.array(sim.pair_potential_str)
    out[f"{tag}/r_cut"] = np.float64(sim.pair_potential_r_cut)
    out[f"{tag}/skin"] = np.float64(sim.neighbor_list_skin)
    out[f"{tag}/kmax"] = np.int32(sim.max_number_of_neighbors)
    if sigma is not None:
        out[f"{tag}/sigma_table"] = np.asarray(sigma, dtype=np.float64)
    if epsilon is not None:
        out[f"{tag}/epsilon_table"] = np.asarray(epsilon, dtype=np.float64)
    if types is not None:
        out[f"{tag}/types"] = np.asarray(types, dtype=np.int32)
    nl = sim.neighbor_list
    counts = np.sum(nl != -1, axis=1)
    out[f"{tag}/nlist"] = nl[:, : max(1, int(counts.max()))].copy()
    out[f"{tag}/forces"] = sim.get_forces()
    try:
        out[f"{tag}/energy"] = np.float64(sim.get_potential_energy())
    except AttributeError:
        # the hard-coded potential returns a Python float beyond r = 1, which has
        # no .astype outside Numba (potential.py:22-23 with :97): no energy here
        pass
    out[f"{tag}/virial"] = np.float64(sim.get_virial())
    out[f"{tag}/laplacian"] = sim.get_laplacian()
    out[f"{tag}/temperature"] = np.float64(sim.get_temperature())
    out[f"{tag}/kinetic_energy"] = np.float64(sim.get_kinetic_energy())
    out[f"{tag}/pressure"] = np.float64(sim.get_pressure())
    if rdf_bins is not None:
        r, g = sim.get_radial_distribution_function(r_bins=rdf_bins)
        out[f"{tag}/rdf_bins"] = rdf_bins
        out[f"{tag}/rdf_r"] = r
        out[f"{tag}/rdf_g"] = g
    print(f"  {tag}: N={sim.positions.shape[0]} D={sim.positions.shape[1]} "
          f"K<={int(counts.max())} ({time.time() - t0:.1f} s)", flush=True)


def make_checkpoint(Simulation):
    """The reference's own ``to_disk`` files for a small seeded 2-D binary
    system with velocities, betas and nonzero images (checkpoint parity)."""
    rng = np.random.default_rng(77)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=((0.0, 0.0),), cells=(4, 3), lattice_constants=(1.0, 1.0))
    n = sim.number_of_particles()
    sim.set_masses(masses=1.0)
    sim.set_types([0, 1] * (n // 2))
    sim.set_density(density=0.9)
    sim.set_pair_potential(pair_potential_str=LJ, r_cut=1.3)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=64)
    sim.set_integrator(time_step=0.002, target_temperature=0.8, temperature_damping_time=0.5)
    sim.velocities = rng.normal(0.0, 0.7, size=sim.positions.shape)
    sim.betas = rng.normal(0.0, 0.05, size=sim.positions.shape)
    sim.masses = rng.uniform(0.5, 2.0, size=(n, 1))
    sim.image_positions = rng.integers(-3, 4, size=sim.positions.shape).astype(np.int32)
    sim.positions = sim.positions + rng.normal(0.0, 0.02, size=sim.positions.shape)
    sim.to_disk(particle_data=os.path.join(HERE, "checkpoint_ref.csv"),
                meta_data=os.path.join(HERE, "checkpoint_ref.toml"))
    print("checkpoint_ref.csv / .toml:", n, "particles")


def make_lammps(Simulation):
    """The reference's ``tools.to_lammps_dump`` text for a small seeded 3-D
    binary system (types, masses, velocities, images, forces), the inputs it
    read, and whether it raises for a 2-D system."""
    from dompap.tools import to_lammps_dump

    rng = np.random.default_rng(91)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=FCC, cells=(2, 2, 2), lattice_constants=(1.0, 1.0, 1.0))
    n = sim.number_of_particles()
    sim.set_masses(masses=1.0)
    sim.set_types([0, 1] * (n // 2))
    sim.set_density(density=0.9)
    sim.set_pair_potential(pair_potential_str=LJ, r_cut=1.5)
    sim.set_neighbor_list(skin=0.3, max_number_of_neighbors=64)
    sim.velocities = rng.normal(0.0, 0.7, size=sim.positions.shape)
    sim.masses = rng.uniform(0.5, 2.0, size=(n, 1))
    sim.image_positions = rng.integers(-3, 4, size=sim.positions.shape).astype(np.int32)
    sim.positions = sim.positions + rng.normal(0.0, 0.02, size=sim.positions.shape)
    sim.number_of_steps = 1234
    forces = sim.get_forces()
    diameters = sim.get_diameters()
    # The tool converts one-element rows with int()/float(), which NumPy 2.5
    # rejects for the (N, 1) arrays the Simulation holds; it is fed the same
    # values as (N,) arrays (what int()/float() of a row returned on the NumPy
    # it was written for).
    from types import SimpleNamespace

    proxy = SimpleNamespace(number_of_steps=sim.number_of_steps, box_vectors=sim.box_vectors,
                            particle_types=sim.particle_types.reshape(-1), masses=sim.masses.reshape(-1),
                            get_diameters=lambda: diameters.reshape(-1), positions=sim.positions,
                            image_positions=sim.image_positions, velocities=sim.velocities,
                            get_forces=lambda: forces)
    text = to_lammps_dump(proxy)
    with open(os.path.join(HERE, "lammps_ref.txt"), "w") as fh:
        fh.write(text)
    np.savez(os.path.join(HERE, "lammps_ref.npz"), positions=sim.positions, velocities=sim.velocities,
             image_positions=sim.image_positions, particle_types=sim.particle_types, masses=sim.masses,
             box_vectors=sim.box_vectors, diameters=diameters, forces=forces,
             number_of_steps=np.int64(sim.number_of_steps))
    sim2 = Simulation()
    sim2.set_positions(unit_cell_coordinates=((0.0, 0.0),), cells=(3, 3), lattice_constants=(1.0, 1.0))
    sim2.set_masses(masses=1.0)
    sim2.set_density(density=0.9)
    sim2.set_pair_potential(pair_potential_str=LJ, r_cut=1.5)
    sim2.set_neighbor_list(skin=0.3, max_number_of_neighbors=64)
    f2 = sim2.get_forces()
    d2 = sim2.get_diameters()
    proxy2 = SimpleNamespace(number_of_steps=0, box_vectors=sim2.box_vectors,
                             particle_types=sim2.particle_types.reshape(-1), masses=sim2.masses.reshape(-1),
                             get_diameters=lambda: d2.reshape(-1), positions=sim2.positions,
                             image_positions=sim2.image_positions, velocities=sim2.velocities,
                             get_forces=lambda: f2)
    try:
        to_lammps_dump(proxy2)
        raised = ""
    except ValueError as exc:
        raised = str(exc)
    with open(os.path.join(HERE, "lammps_ref_2d_error.txt"), "w") as fh:
        fh.write(raised)
    print("lammps_ref.txt:", n, "particles; 2-D raises:", repr(raised))


def make_rdf_types(rpos):
    """Per-type g(r) of the binary (Wahnstrom-type) configuration already in
    ``golden_configs.npz`` (``wahn``): the reference's
    ``positions.get_radial_distribution_function(positions_a, positions_b, box,
    r_bins)`` on the type subsets A-A, A-B and B-B, as a ``Simulation`` user
    computes the g(r) of each pair type."""
    cfg = np.load(os.path.join(HERE, "golden_configs.npz"))
    pos = cfg["wahn/positions"]
    box = cfg["wahn/box"]
    types = cfg["wahn/types"].reshape(-1)
    bins = np.linspace(0.5, 3.5, 61)
    out = {"bins": bins}
    for a, b, key in ((0, 0, "AA"), (0, 1, "AB"), (1, 1, "BB")):
        r, g = rpos.get_radial_distribution_function(pos[types == a], pos[types == b], box, bins)
        out[f"{key}/r"] = r
        out[f"{key}/g"] = g
    np.savez_compressed(os.path.join(HERE, "golden_rdf_types.npz"), **out)
    print("golden_rdf_types.npz:", {k: float(np.max(out[k + "/g"])) for k in ("AA", "AB", "BB")})


def make_methods(Simulation):
    """The reference's own double-loop and vectorised force and energy
    methods (dompap/potential.py:103-160,191-250,298-324, dispatched by
    Simulation.get_forces / get_potential_energy) on configurations already in
    ``golden_configs.npz``, rebuilt through the public setters: ``callable``
    (asymmetric epsilon(n, m): the methods differ), ``wahn`` (per-type table)
    and ``harm2d``."""
    cfg = np.load(os.path.join(HERE, "golden_configs.npz"))
    out = {}
    for tag in ("callable", "wahn", "harm2d"):
        c = {k.split("/", 1)[1]: cfg[k] for k in cfg.files if k.startswith(tag + "/")}
        pos = np.array(c["positions"])
        n, dim = pos.shape
        sim = Simulation()
        sim.positions = pos
        sim.box_vectors = np.array(c["box"])
        sim.velocities = np.array(c["velocities"])
        sim.betas = np.zeros((n, dim))
        sim.image_positions = np.zeros((n, dim), dtype=np.int32)
        sim.masses = np.array(c["masses"]).reshape(-1, 1)
        sim.particle_types = np.zeros((n, 1), dtype=np.int32)
        sim.set_pair_potential(pair_potential_str=str(c["pot"]), r_cut=float(c["r_cut"]))
        if "types" in c:
            t, st, et = c["types"].reshape(-1), c["sigma_table"], c["epsilon_table"]
            sim.set_pair_potential_parameters(sigma=lambda a, b: st[t[a], t[b]], epsilon=lambda a, b: et[t[a], t[b]])
        elif "sigma_table" in c and np.ndim(c["sigma_table"]) == 2:
            sm, em = c["sigma_table"], c["epsilon_table"]
            sim.set_pair_potential_parameters(sigma=lambda a, b: sm[a, b], epsilon=lambda a, b: em[a, b])
        sim.set_neighbor_list(skin=float(c["skin"]), max_number_of_neighbors=int(c["kmax"]))
        for method in ("neighbor list", "double loop", "double loop single core", "vectorized"):
            sim.force_method_str = method
            out[f"{tag}/forces/{method}"] = np.array(sim.get_forces())
        for method in ("neighbor list", "double loop", "double loop single core"):
            sim.energy_method_str = method
            out[f"{tag}/energy/{method}"] = np.float64(sim.get_potential_energy())
        print(f"  {tag}: N={n}", flush=True)
    np.savez_compressed(os.path.join(HERE, "golden_methods.npz"), **out)
    print("golden_methods.npz:", len(out), "arrays")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("DOMPAP_REFERENCE"),
                    required="DOMPAP_REFERENCE" not in os.environ, help="path of an unmodified dompap 0.0.6 source tree (or set DOMPAP_REFERENCE)")
    ap.add_argument("--only", choices=["checkpoint", "lammps", "rdf_types", "methods"], default=None,
                    help="regenerate only the named fixture")
    args = ap.parse_args()
    dompap = import_reference(args.reference)
    if args.only == "checkpoint":
        from dompap import Simulation

        make_checkpoint(Simulation)
        return
    if args.only == "lammps":
        from dompap import Simulation

        make_lammps(Simulation)
        return
    if args.only == "methods":
        from dompap import Simulation

        make_methods(Simulation)
        return
    if args.only == "rdf_types":
        from dompap import positions as rpos

        make_rdf_types(rpos)
        return
    from dompap import Simulation
    from dompap import neighbor_list as rnl
    from dompap import potential as rpot
    from dompap import positions as rpos
    from dompap import integrator as rint

    # ---------------- the reference's own unit-test inputs ----------------
    unit = {}
    p3 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [2, 2, 2], [5, 5, 0]], dtype=np.float64)
    p2 = np.array([[0, 0], [1, 0], [0, 1], [2, 2], [5, 5]], dtype=np.float64)
    unit["nl3d/positions"] = p3
    unit["nl3d/nlist"] = rnl.get_neighbor_list_double_loop(p3, np.array([6.0] * 3), np.float64(1.5), 4)
    unit["nl2d/positions"] = p2
    unit["nl2d/nlist"] = rnl.get_neighbor_list_double_loop(p2, np.array([6.0] * 2), np.float64(1.5), 4)
    # skin trigger around skin/2 (tests/test_neighbor_list.py:94-118 inputs)
    skins = np.concatenate([np.linspace(0.01, 0.99, 10), np.linspace(1.01, 1.5, 10)])
    pos = np.array([[0, 0, 0], [1, 1, 1]], dtype=np.float64)
    old = np.array([[0.5, 0, 0], [1, 1, 1]], dtype=np.float64)
    unit["skin/skins"] = skins
    unit["skin/is_old"] = np.array([rnl.neighbor_list_is_old(pos, old, np.array([5.0] * 3), s) for s in skins])
    # potentials at sample points
    rr = np.linspace(0.85, 3.2, 41)
    for tag, s, rc in (("harm", "(1-r)**2", 1.0), ("lj", LJ, 2.5), ("ljinf", LJ, np.inf), ("exp", EXPENSIVE, 3.0)):
        u, f, c = rpot.make_pair_potential(s, rc)
        unit[f"pot_{tag}/r"] = rr
        unit[f"pot_{tag}/u"] = np.array([float(u(x)) for x in rr])
        unit[f"pot_{tag}/f"] = np.array([float(f(x)) for x in rr])
        unit[f"pot_{tag}/c"] = np.array([float(c(x)) for x in rr])
    unit["pot_exp/expr"] = np.array(EXPENSIVE)
    # hard-coded 'Harmonic repulsive'
    _, hu, hf, hc, hrc = rpot.hardcoded_pair_potentials["Harmonic repulsive"]
    unit["pot_hard/r"] = rr
    unit["pot_hard/u"] = np.array([hu(x) for x in rr])
    unit["pot_hard/f"] = np.array([hf(x) for x in rr])
    # wrap into box (tests/test_positions.py:78-93 inputs)
    wp = np.array([[0.1, 0.1, 0.1], [2.5, 2.5, 2.5], [-0.1, -0.1, -0.1]], dtype=np.float64)
    wi = np.zeros(wp.shape, dtype=np.int32)
    unit["wrap/in"] = wp.copy()
    rpos.wrap_into_box(wp, wi, np.array([2.0] * 3))
    unit["wrap/positions"] = wp
    unit["wrap/images"] = wi
    # G-JF with a recorded normal stream (integrator.py:30 draws np.random.normal)
    rng = np.random.default_rng(7)
    gp = rng.uniform(0, 5, size=(64, 3))
    gv = rng.normal(size=(64, 3))
    gb = rng.normal(scale=0.1, size=(64, 3))
    gf = rng.normal(size=(64, 3))
    gm = rng.uniform(0.5, 2.0, size=(64, 1))
    np.random.seed(1234)
    normals = np.random.normal(0, 1, gv.shape)
    np.random.seed(1234)
    npos, nvel, nbeta = rint.make_one_step(gp, gv, gb, gf, gm, np.float64(0.005), np.float64(1.3), np.float64(0.1))
    for k, v in dict(positions=gp, velocities=gv, betas=gb, forces=gf, masses=gm, normals=normals,
                     new_positions=npos, new_velocities=nvel, new_betas=nbeta).items():
        unit[f"gjf/{k}"] = v
    lp, lv = rint.make_one_step_leap_frog(gp, gv, gf, gm, np.float64(0.005))
    unit["leapfrog/new_positions"] = lp
    unit["leapfrog/new_velocities"] = lv
    # doctest values of Simulation.py
    sim = Simulation()
    sim.scale_box(0.5)
    unit["doctest/energy_scaled"] = np.float64(sim.get_potential_energy())  # :553-555
    sim = Simulation()
    sim.positions[0] = [0.5, 0.0, 0.0]
    unit["doctest/force0"] = sim.get_forces()[0]  # :602-605
    sim = Simulation()
    unit["doctest/laplacian0"] = np.float64(sim.get_laplacian()[0])  # :1213-1215
    # sigma=2, epsilon=4 semantics (tests/test_potential.py:81-140 inputs)
    sim = Simulation()
    sim.positions = np.array([[0, 0, 0], [1, 0, 0]], dtype=np.float64)
    sim.box_vectors = np.array([3.0, 3.0, 3.0])
    sim.velocities = np.zeros((2, 3))
    sim.betas = np.zeros((2, 3))
    sim.image_positions = np.zeros((2, 3), dtype=np.int32)
    sim.masses = np.ones((2, 1))
    sim.particle_types = np.zeros((2, 1), dtype=np.int32)
    sim.set_pair_potential("(1-r)**2", 1.0)
    sim.set_pair_potential_parameters(sigma=2.0, epsilon=4.0)
    unit["sig2eps4/energy"] = np.float64(sim.get_potential_energy())
    unit["sig2eps4/forces"] = sim.get_forces()
    np.savez_compressed(os.path.join(HERE, "golden_unit.npz"), **unit)
    print("golden_unit.npz:", len(unit), "arrays")

    # ---------------- seeded configurations through Simulation ----------------
    cfg = {}
    rng = np.random.default_rng(20240601)
    # LJ fcc 5^3 = 500 at 0.8442, r_cut 2.5, skin 0.5 (the N=500 LJ case)
    sim = build_sim(Simulation, FCC, (5, 5, 5), 0.8442, LJ, 2.5, 0.5, rng, jitter=0.03)
    record_sim(cfg, "lj500", sim, rdf_bins=np.linspace(0.5, 4.0, 36))
    # harmonic (1-r)^2, compressed so forces are non-zero, D = 2, 3, 4
    sim = build_sim(Simulation, FCC, (4, 4, 4), 1.5, "(1-r)**2", 1.0, 0.2, rng, jitter=0.02)
    record_sim(cfg, "harm3d", sim)
    sim = build_sim(Simulation, ((0.0, 0.0),), (16, 16), 1.3, "(1-r)**2", 1.0, 0.2, rng, jitter=0.02)
    record_sim(cfg, "harm2d", sim)
    sim = build_sim(Simulation, ((0.0, 0.0, 0.0, 0.0),), (5, 5, 5, 5), 1.4, "(1-r)**2", 1.0, 0.2, rng, jitter=0.02)
    record_sim(cfg, "harm4d", sim)
    # hard-coded harmonic potential
    sim = build_sim(Simulation, FCC, (4, 4, 4), 1.5, "Harmonic repulsive", 1.0, 0.2, rng, jitter=0.02)
    record_sim(cfg, "hard3d", sim)
    # sigma = 2, epsilon = 4 on many pairs (no 1/sigma factor)
    sim = build_sim(Simulation, FCC, (4, 4, 4), 0.2, "(1-r)**2", 1.0, 0.3, rng, jitter=0.05)
    sim.set_pair_potential_parameters(sigma=2.0, epsilon=4.0)
    record_sim(cfg, "sig2eps4", sim, sigma=2.0, epsilon=4.0)
    # Wahnstrom-type binary LJ: sigma/epsilon from a type table through index callables
    sim = build_sim(Simulation, ((0.0, 0.0, 0.0),), (8, 8, 8), 0.75, LJ, 2.5, 0.5, rng, jitter=0.03)
    types = np.zeros(sim.positions.shape[0], dtype=np.int32)
    types[rng.permutation(types.size)[: types.size // 2]] = 1
    sig_t = np.array([[1.0, 1.1], [1.1, 1.2]])
    eps_t = np.array([[1.0, 1.0], [1.0, 1.0]])
    sim.set_types(types=[int(t) for t in types])
    sim.set_masses(masses=[2.0 if t == 0 else 1.0 for t in types])
    sim.set_pair_potential_parameters(sigma=lambda n, m: sig_t[types[n], types[m]],
                                      epsilon=lambda n, m: eps_t[types[n], types[m]])
    record_sim(cfg, "wahn", sim, sigma=sig_t, epsilon=eps_t, types=types)
    # index callable that is not a type table (n == m special case, as in the Simulation docstring)
    sim = build_sim(Simulation, FCC, (3, 3, 3), 1.2, "(1-r)**2", 1.0, 0.3, rng, jitter=0.03)
    nn = sim.positions.shape[0]
    sig_m = np.where(np.eye(nn, dtype=bool), 1.0, 1.2)
    eps_m = np.where(np.eye(nn, dtype=bool), 1.0, 0.5) + 0.001 * (np.arange(nn)[:, None] % 3)
    sim.set_pair_potential_parameters(sigma=lambda n, m: sig_m[n, m], epsilon=lambda n, m: eps_m[n, m])
    record_sim(cfg, "callable", sim, sigma=sig_m, epsilon=eps_m)
    # the expensive potential, smoothly shifted at 3.0
    sim = build_sim(Simulation, FCC, (4, 4, 4), 0.8, EXPENSIVE, 3.0, 0.3, rng, jitter=0.03)
    record_sim(cfg, "expensive", sim)
    np.savez_compressed(os.path.join(HERE, "golden_configs.npz"), **cfg)
    print("golden_configs.npz:", len(cfg), "arrays")

    # ---------------- deterministic trajectories ----------------
    traj = {}
    # NVE leap-frog, 12 steps of the LJ N=500 case
    rng = np.random.default_rng(99)
    sim = build_sim(Simulation, FCC, (5, 5, 5), 0.8442, LJ, 2.5, 0.3, rng, jitter=0.03)
    sim.velocities = rng.normal(0.0, 1.0, size=sim.positions.shape)
    sim.set_integrator(time_step=0.005)
    traj["nve/positions0"] = sim.positions.copy()
    traj["nve/velocities0"] = sim.velocities.copy()
    traj["nve/images0"] = sim.image_positions.copy()
    traj["nve/box"] = sim.box_vectors.copy()
    steps = 12
    for _ in range(steps):
        sim.step_leap_frog()
    traj["nve/steps"] = np.int32(steps)
    traj["nve/positions"] = sim.positions.copy()
    traj["nve/velocities"] = sim.velocities.copy()
    traj["nve/images"] = sim.image_positions.copy()
    traj["nve/energy"] = np.float64(sim.get_potential_energy())
    # G-JF with tau = inf (the random term is multiplied by sqrt(0)): deterministic
    rng = np.random.default_rng(5)
    sim = build_sim(Simulation, FCC, (4, 4, 4), 1.5, "(1-r)**2", 1.0, 0.2, rng, jitter=0.02)
    sim.velocities = rng.normal(0.0, 0.3, size=sim.positions.shape)
    sim.set_integrator(time_step=0.01, target_temperature=0.5, temperature_damping_time=np.inf)
    traj["gjfinf/positions0"] = sim.positions.copy()
    traj["gjfinf/velocities0"] = sim.velocities.copy()
    traj["gjfinf/images0"] = sim.image_positions.copy()
    traj["gjfinf/box"] = sim.box_vectors.copy()
    for _ in range(10):
        sim.step()
    traj["gjfinf/steps"] = np.int32(10)
    traj["gjfinf/positions"] = sim.positions.copy()
    traj["gjfinf/velocities"] = sim.velocities.copy()
    traj["gjfinf/images"] = sim.image_positions.copy()
    np.savez_compressed(os.path.join(HERE, "golden_traj.npz"), **traj)
    print("golden_traj.npz:", len(traj), "arrays")
    make_checkpoint(Simulation)


if __name__ == "__main__":
    main()
