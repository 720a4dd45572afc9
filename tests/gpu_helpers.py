"""Helpers shared by the GPU tests: build a ``dompap_gb300.Simulation`` from a
golden configuration, exactly as the fixture generator built the reference one."""
import numpy as np

from conftest import config_of
from oracle import numpy_ref as ref


def sim_from_config(cfg, tag, method="double loop", precision="fp64"):
    from dompap_gb300 import Simulation

    sim = Simulation(precision=precision)
    n, d = cfg["positions"].shape
    sim.box_vectors = cfg["box"]
    sim.positions = cfg["positions"]
    sim.velocities = cfg["velocities"]
    sim.betas = np.zeros((n, d))
    sim.image_positions = np.zeros((n, d), dtype=np.int32)
    sim.masses = cfg["masses"]
    if "types" in cfg:
        sim.set_types([int(t) for t in cfg["types"]])
    else:
        sim.particle_types = np.zeros((n, 1), dtype=np.int32)
    pot = "Harmonic repulsive" if tag == "hard3d" else str(cfg["pot"])
    sim.set_pair_potential(pair_potential_str=pot, r_cut=float(cfg["r_cut"]))
    if "types" in cfg:
        types = cfg["types"]
        st, et = cfg["sigma_table"], cfg["epsilon_table"]
        sim.set_pair_potential_parameters(sigma=lambda a, b: st[types[a], types[b]],
                                          epsilon=lambda a, b: et[types[a], types[b]])
    elif "sigma_table" in cfg and np.ndim(cfg["sigma_table"]) == 2:
        sm, em = cfg["sigma_table"], cfg["epsilon_table"]
        sim.set_pair_potential_parameters(sigma=lambda a, b: sm[a, b], epsilon=lambda a, b: em[a, b])
    elif "sigma_table" in cfg:
        sim.set_pair_potential_parameters(sigma=float(cfg["sigma_table"]), epsilon=float(cfg["epsilon_table"]))
    sim.set_neighbor_list(skin=float(cfg["skin"]), max_number_of_neighbors=int(cfg["kmax"]), method_str=method)
    return sim


def oracle_params(cfg):
    n = cfg["positions"].shape[0]
    if "types" in cfg:
        t = cfg["types"]
        return cfg["sigma_table"][t[:, None], t[None, :]], cfg["epsilon_table"][t[:, None], t[None, :]]
    sig = cfg.get("sigma_table", np.float64(1.0))
    eps = cfg.get("epsilon_table", np.float64(1.0))
    return (float(sig) if np.ndim(sig) == 0 else sig), (float(eps) if np.ndim(eps) == 0 else eps)


def oracle_potential(cfg, tag):
    if tag == "hard3d":
        u, f, c, _ = ref.harmonic_repulsive()
        return u, f, c
    return ref.make_pair_potential(str(cfg["pot"]), float(cfg["r_cut"]))


def rel_rms(got, want):
    den = np.sqrt(np.mean(np.asarray(want) ** 2))
    num = np.sqrt(np.mean((np.asarray(got) - np.asarray(want)) ** 2))
    return num / den if den > 0 else num


__all__ = ["sim_from_config", "oracle_params", "oracle_potential", "rel_rms", "config_of"]
