"""Checkpoint files (dompap/Simulation.py:1019-1203) against the reference's
own ``to_disk`` output (``tests/golden/checkpoint_ref.*``, written by
``make_golden.py``): the particle CSV is reproduced byte for byte, the
metadata parses to the same values, and a GPU system restored from the
reference's files reproduces the observables the reference wrote."""
import os
import tomllib

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CSV = os.path.join(GOLDEN, "checkpoint_ref.csv")
TOML = os.path.join(GOLDEN, "checkpoint_ref.toml")


class _HostState:
    """The attributes and observables ``io.to_disk``/``io.from_disk`` use,
    without a device (the observables return the reference's values)."""

    def __init__(self, meta):
        self._meta = meta
        self.pair_potential_str = meta["pair_potential_str"]
        self.pair_potential_r_cut = meta["pair_potential_r_cut"]
        self.neighbor_list_skin = meta["neighbor_list_skin"]
        self.max_number_of_neighbors = meta["max_number_of_neighbors"]
        self.neighbor_list_method_str = meta["neighbor_list_method_str"]
        self.energy_method_str = meta["energy_method_str"]
        self.force_method_str = meta["force_method_str"]
        self.time_step = meta["time_step"]
        self.temperature_target = meta["temperature_target"]
        self.temperature_damping_time = meta["temperature_damping_time"]
        self.number_of_steps = meta["number_of_steps"]
        self.number_of_neighbor_list_updates = meta["number_of_neighbor_list_updates"]

    def get_dimensions_of_space(self):
        return self.positions.shape[1]

    def number_of_particles(self):
        return self.positions.shape[0]

    def __getattr__(self, name):
        key = {"get_temperature": "temperature", "get_potential_energy": "potential_energy",
               "get_kinetic_energy": "kinetic_energy", "get_pressure": "pressure", "get_virial": "virial",
               "get_density": "density", "get_volume": "volume"}.get(name)
        if key is None:
            raise AttributeError(name)
        return lambda: self._meta[key]


def _reference_meta():
    with open(TOML, "rb") as fh:
        return tomllib.load(fh)


def test_csv_round_trip_is_byte_identical(tmp_path):
    from dompap_gb300 import io

    meta = _reference_meta()
    st = _HostState(meta)
    got_meta = io.from_disk(st, particle_data=CSV, meta_data=TOML, set_only_particle_data=True)
    assert got_meta == meta
    assert st.positions.shape == (12, 2) and st.image_positions.dtype == np.int32
    out_csv, out_toml = tmp_path / "c.csv", tmp_path / "c.toml"
    io.to_disk(st, particle_data=str(out_csv), meta_data=str(out_toml))
    assert out_csv.read_bytes() == open(CSV, "rb").read()
    with open(out_toml, "rb") as fh:
        assert tomllib.load(fh) == meta


def test_from_disk_rejects_unknown_columns(tmp_path):
    from dompap_gb300 import io

    bad = tmp_path / "bad.csv"
    bad.write_text("ptype,mass,pos_0,pos_1,spin_0\n0,1.0,0.1,0.2,1\n")
    with pytest.raises(ValueError):
        io.from_disk(_HostState(_reference_meta()), particle_data=str(bad), meta_data=TOML,
                     set_only_particle_data=True)


@pytest.mark.gpu
def test_restored_system_reproduces_reference_observables(tmp_path):
    from dompap_gb300 import Simulation

    meta = _reference_meta()
    sim = Simulation()
    sim.from_disk(particle_data=CSV, meta_data=TOML)
    assert sim.number_of_particles() == 12
    # float64-parity pair sums: the reference's values to 1e-10 of their pair-term scale
    assert abs(sim.get_potential_energy() - meta["potential_energy"]) <= 1e-10 * max(1.0, abs(meta["potential_energy"]))
    assert abs(sim.get_virial() - meta["virial"]) <= 1e-10 * max(1.0, abs(meta["virial"]))
    assert abs(sim.get_pressure() - meta["pressure"]) <= 1e-10 * abs(meta["pressure"])
    assert abs(sim.get_temperature() - meta["temperature"]) <= 1e-13 * meta["temperature"]
    assert abs(sim.get_kinetic_energy() - meta["kinetic_energy"]) <= 1e-13 * meta["kinetic_energy"]
    out_csv, out_toml = tmp_path / "c.csv", tmp_path / "c.toml"
    sim.to_disk(particle_data=str(out_csv), meta_data=str(out_toml))
    assert out_csv.read_bytes() == open(CSV, "rb").read()


@pytest.mark.parametrize("dim", [3, 4])
def test_round_trip_other_dimensions(tmp_path, dim):
    """to_disk -> from_disk restores positions, images, velocities, betas,
    types and masses exactly in 3 and 4 dimensions (the format's columns
    follow the dimension, dompap/Simulation.py:1019-1203)."""
    from dompap_gb300 import io

    rng = np.random.default_rng(dim)
    n = 17
    meta = _reference_meta()
    st = _HostState(meta)
    st.positions = rng.uniform(0.0, 5.0, size=(n, dim))
    st.image_positions = rng.integers(-4, 5, size=(n, dim)).astype(np.int32)
    st.velocities = rng.normal(size=(n, dim))
    st.betas = rng.normal(scale=0.1, size=(n, dim))
    st.particle_types = rng.integers(0, 3, size=(n, 1)).astype(np.int32)
    st.masses = rng.uniform(0.5, 2.0, size=(n, 1))
    st.box_vectors = np.full(dim, 5.0)
    csv, toml = tmp_path / "s.csv", tmp_path / "s.toml"
    io.to_disk(st, particle_data=str(csv), meta_data=str(toml))
    back = _HostState(meta)
    io.from_disk(back, particle_data=str(csv), meta_data=str(toml), set_only_particle_data=True)
    for name in ("positions", "image_positions", "velocities", "betas", "particle_types", "masses"):
        assert np.array_equal(np.asarray(getattr(back, name)).reshape(getattr(st, name).shape), getattr(st, name)), name


def test_toml_float_format_matches_toml_package():
    """dompap writes its metadata with the ``toml`` package, whose floats drop
    a leading zero of the exponent (``time_step = 1e-5``); values round-trip."""
    from dompap_gb300.io import _toml_value

    assert _toml_value(1e-05) == "1e-5"
    assert _toml_value(2.5e-07) == "2.5e-7"
    assert _toml_value(1e20) == "1e+20"
    assert _toml_value(1.5e+300) == "1.5e+300"
    assert _toml_value(0.002) == "0.002"
    for v in (1e-05, 2.5e-07, 1e20, 0.002, 123456.789):
        assert tomllib.loads(f"x = {_toml_value(v)}\n")["x"] == v
