"""Checkpoint files in dompap's format (dompap/Simulation.py:1019-1203).

``to_disk`` writes the particle CSV (``ptype,mass,pos_d..,vel_d..,imgpos_d..,
beta_d..``) byte for byte as dompap does, and the TOML metadata with dompap's
keys and values in the ``toml`` package's flat form (floats with a one-digit
exponent where it can: 1e-5); the state is copied from the GPU first. ``from_disk`` reads both, replaces the system and re-applies
the potential, neighbour list and integrator, so a GPU run resumes from a
dompap checkpoint and vice versa.
"""
from __future__ import annotations

import os
import tomllib

import numpy as np


def _toml_value(value):
    if isinstance(value, bool):
        return "true" if value else "false"
    if isinstance(value, str):
        return '"' + value.replace("\\", "\\\\").replace('"', '\\"') + '"'
    if isinstance(value, (list, tuple)):
        return "[ " + ", ".join(_toml_value(v) for v in value) + ",]"
    if isinstance(value, float):
        if not np.isfinite(value):
            return "inf" if value > 0 else ("-inf" if value < 0 else "nan")
        # the toml package prints floats with str() and drops a leading zero of
        # the exponent (1e-05 -> 1e-5)
        return repr(value).replace("e+0", "e+").replace("e-0", "e-")
    return repr(value)


def to_disk(sim, particle_data="simulation.csv", meta_data="simulation.toml") -> None:
    """Particle CSV and TOML metadata as dompap writes them
    (dompap/Simulation.py:1019-1079); the CSV is byte-identical."""
    dims = sim.get_dimensions_of_space()
    types = sim.particle_types
    masses = sim.masses
    pos = sim.positions
    vel = sim.velocities
    img = sim.image_positions
    betas = sim.betas
    header = "ptype,mass"
    for prefix in ("pos", "vel", "imgpos", "beta"):
        for d in range(dims):
            header += f",{prefix}_{d}"
    rows = []
    for n in range(sim.number_of_particles()):
        cols = [f"{types[n, 0]}", f"{masses[n, 0]}"]
        cols += [f"{pos[n, d]}" for d in range(dims)]
        cols += [f"{vel[n, d]}" for d in range(dims)]
        cols += [f"{img[n, d]}" for d in range(dims)]
        cols += [f"{betas[n, d]}" for d in range(dims)]
        rows.append(",".join(cols))
    with open(particle_data, "w") as fh:
        fh.write(header + "".join("\n" + r for r in rows) + "\n")
    meta = {
        "box_vectors": [float(b) for b in sim.box_vectors],
        "dimensions_of_space": dims,
        "number_of_particles": sim.number_of_particles(),
        "temperature": sim.get_temperature(),
        "potential_energy": sim.get_potential_energy(),
        "kinetic_energy": sim.get_kinetic_energy(),
        "pressure": sim.get_pressure(),
        "virial": sim.get_virial(),
        "density": sim.get_density(),
        "volume": sim.get_volume(),
        "pair_potential_str": sim.pair_potential_str,
        "pair_potential_r_cut": float(sim.pair_potential_r_cut),
        "neighbor_list_skin": float(sim.neighbor_list_skin),
        "max_number_of_neighbors": int(sim.max_number_of_neighbors),
        "neighbor_list_method_str": sim.neighbor_list_method_str,
        "energy_method_str": sim.energy_method_str,
        "force_method_str": sim.force_method_str,
        "time_step": float(sim.time_step),
        "temperature_target": float(sim.temperature_target),
        "temperature_damping_time": float(sim.temperature_damping_time),
        "number_of_steps": int(sim.number_of_steps),
        "number_of_neighbor_list_updates": int(sim.number_of_neighbor_list_updates),
    }
    with open(meta_data, "w") as fh:
        fh.write("".join(f"{k} = {_toml_value(v)}\n" for k, v in meta.items()) + "\n")


def from_disk(sim, particle_data="simulation.csv", meta_data="simulation.toml", verbose=False,
              set_only_particle_data=False) -> dict:
    """Read dompap's checkpoint files (dompap/Simulation.py:1081-1203) into
    ``sim``; returns the metadata."""
    if not os.path.isfile(particle_data):
        raise FileNotFoundError(f"File not found: {particle_data}")
    if not os.path.isfile(meta_data):
        raise FileNotFoundError(f"File not found: {meta_data}")
    with open(meta_data, "rb") as fh:
        meta = tomllib.load(fh)
    box = np.array(meta["box_vectors"], dtype=np.float64)
    dims = box.shape[0]
    n = int(meta["number_of_particles"])
    if verbose:
        print(f"Dimensions of space: {sim.get_dimensions_of_space()} -> {dims}")
        print(f"number_of_particles: {sim.number_of_particles()} -> {n}")
    types = np.zeros((n, 1), dtype=np.int32)
    masses = np.zeros((n, 1), dtype=np.float64)
    pos = np.zeros((n, dims), dtype=np.float64)
    vel = np.zeros((n, dims), dtype=np.float64)
    img = np.zeros((n, dims), dtype=np.int32)
    betas = np.zeros((n, dims), dtype=np.float64)
    with open(particle_data) as fh:
        lines = [ln for ln in fh.read().splitlines()]
    names = lines[0].split(",")
    body = [ln for ln in lines[1:] if ln.strip()]
    for i, line in enumerate(body):
        for value, name in zip(line.split(","), names):
            if "_" in name:
                kind, d = name.split("_")
                d = int(d)
                if kind == "pos":
                    pos[i, d] = float(value)
                elif kind == "vel":
                    vel[i, d] = float(value)
                elif kind == "imgpos":
                    img[i, d] = int(value)
                elif kind == "beta":
                    betas[i, d] = float(value)
                else:
                    raise ValueError(f"Unknown column name: {kind}")
            elif name == "ptype":
                types[i, 0] = int(value)
            elif name == "mass":
                masses[i, 0] = float(value)
            else:
                raise ValueError(f"Unknown column name: {name}")
    sim.box_vectors = box
    sim.particle_types = types
    sim.positions = pos
    sim.velocities = vel
    sim.image_positions = img
    sim.betas = betas
    sim.masses = masses
    if not set_only_particle_data:
        sim.set_pair_potential(pair_potential_str=meta["pair_potential_str"], r_cut=meta["pair_potential_r_cut"],
                               force_method=meta["force_method_str"], energy_method=meta["energy_method_str"])
        sim.set_neighbor_list(skin=meta["neighbor_list_skin"], max_number_of_neighbors=meta["max_number_of_neighbors"],
                              method_str=meta["neighbor_list_method_str"])
        sim.set_integrator(time_step=meta["time_step"], target_temperature=meta["temperature_target"],
                           temperature_damping_time=meta["temperature_damping_time"])
        sim.number_of_steps = meta["number_of_steps"]
        sim.number_of_neighbor_list_updates = meta["number_of_neighbor_list_updates"]
    return meta
