"""Thousands of independent replicas advanced by one persistent GPU kernel.

A Python loop of ``Simulation.run`` over many small systems is launch-bound
(dompap/Simulation.py:726-737 runs one system at a time). ``Replicas`` keeps
every replica resident on the GPU and advances all of them with one
persistent kernel per ``run`` (captured in a CUDA graph): each CTA takes a
replica from a work queue, largest first, and runs all steps of it with the
replica's positions in shared memory and its Verlet list (partners within
r_cut + skin, rebuilt when a particle moved more than skin/2) in HBM. Pair
forces are float32 (from fixed-point displacements, ~1e-7 relative),
integration, wrap and observables float64; sigma = epsilon = 1.

The launch shape (threads per CTA for small and large replicas and the size
split between them) is picked by ``autotune``, which times short runs of the
candidates on the actual batch.
"""
from __future__ import annotations

import ctypes
import itertools
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import codegen
from .positions import FCC, generate_positions


@dataclass
class ReplicaSpec:
    """One independent system of a batch: its lattice, velocities, box and
    Langevin target temperature."""

    positions: np.ndarray   # (N, D), inside [0, L)
    velocities: np.ndarray  # (N, D)
    box: np.ndarray         # (D,)
    temperature: float


class Replicas:
    """Thousands of independent systems of one pair potential (uneven N and
    temperature) advanced together by one persistent kernel per run; each
    replica follows dompap's step (dompap/Simulation.py:681-737) with float32
    pair forces and float64 integration."""

    def __init__(self, specs: list[ReplicaSpec], pair_potential_str: str, r_cut: float, time_step: float = 0.005,
                 damping_time: float = 0.1, mass: float = 1.0, seed: int | None = None, skin: float = 0.45,
                 max_number_of_neighbors: int = 0):
        if not specs:
            raise ValueError("need at least one replica")
        self.dim = int(specs[0].positions.shape[1])
        self.counts = np.array([s.positions.shape[0] for s in specs], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)])
        self.n_rep = len(specs)
        self.ntot = int(self.offsets[-1])
        self.boxes = np.array([np.asarray(s.box, dtype=np.float64) for s in specs])
        self.temperatures = np.array([float(s.temperature) for s in specs])
        for s in specs:
            if s.positions.shape[1] != self.dim:
                raise ValueError("all replicas must have the same dimension")
            if np.min(s.box) < 2 * r_cut:
                raise ValueError("a replica box is shorter than 2 r_cut (single-image convention)")
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.dp_batch_create(self.dim, self.n_rep, _lib.iptr(np.ascontiguousarray(self.counts)),
                                       ctypes.byref(h)))
        self._h = h
        pos = np.ascontiguousarray(np.concatenate([s.positions for s in specs]), dtype=np.float64)
        vel = np.ascontiguousarray(np.concatenate([s.velocities for s in specs]), dtype=np.float64)
        _lib.check(lib.dp_batch_set_state(h, _lib.dptr(pos), _lib.dptr(vel),
                                          _lib.dptr(np.ascontiguousarray(self.boxes)),
                                          _lib.dptr(np.ascontiguousarray(self.temperatures))))
        src, rc = codegen.make_pair_source(pair_potential_str, r_cut)
        self.r_cut = rc
        self.pair_potential_str = pair_potential_str
        _lib.check(lib.dp_batch_set_potential(h, src.encode(), rc))
        seed = int(np.random.randint(0, 2**62)) if seed is None else int(seed)
        _lib.check(lib.dp_batch_set_integrator(h, float(time_step), float(damping_time), float(mass), seed))
        self.time_step, self.damping_time, self.mass = time_step, damping_time, mass
        self.set_neighbor_list(skin, max_number_of_neighbors)
        self.set_launch(1024, 256, 512)

    # ---------------------------------------------------------------- running
    def set_neighbor_list(self, skin: float = 0.45, max_number_of_neighbors: int = 0) -> None:
        """Verlet lists per replica with partners within r_cut + skin (skin < 0:
        the 27-cell stencil every step); max_number_of_neighbors = 0 sizes them
        from the densest replica (a given capacity is rounded up to a multiple
        of 8: the lists are stored in 8-entry chunks)."""
        _lib.check(_lib.load().dp_batch_set_neighbor_list(self._h, float(skin), int(max_number_of_neighbors)))
        self.skin = skin

    def list_stats(self) -> dict:
        """Verlet-list builds so far, replicas that overflowed their list (and
        used the cell stencil), and the list capacity per particle."""
        b, o, k = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int32(0)
        _lib.check(_lib.load().dp_batch_list_stats(self._h, ctypes.byref(b), ctypes.byref(o), ctypes.byref(k)))
        return {"builds": int(b.value), "overflowed": int(o.value), "kmax": int(k.value)}

    def set_launch(self, split_n: int, threads_small: int, threads_large: int) -> None:
        """Launch shape: replicas of up to ``split_n`` particles run in CTAs of
        ``threads_small`` threads, larger ones in CTAs of ``threads_large``."""
        _lib.check(_lib.load().dp_batch_set_launch(self._h, int(split_n), int(threads_small), int(threads_large)))
        self.launch = (split_n, threads_small, threads_large)

    def run(self, steps: int, sample_every: int = 0, nve: bool = False, record_forces: bool = False) -> float:
        """Advance every replica ``steps`` steps; returns the device time in ms."""
        ms = ctypes.c_float(0.0)
        _lib.check(_lib.load().dp_batch_run(self._h, int(steps), int(sample_every), int(bool(nve)),
                                            int(bool(record_forces)), ctypes.byref(ms)))
        return float(ms.value)

    def autotune(self, steps: int = 10, candidates=None, verbose: bool = False):
        """Pick the launch shape with the shortest device time of ``steps`` steps
        (each candidate timed twice, the first run being a warm-up). The state
        advances by those steps."""
        if candidates is None:
            candidates = [(s, ts, tl) for s, ts, tl in itertools.product((512, 1024, 2048), (128, 256), (256, 512))]
        best = None
        for cand in candidates:
            try:
                self.set_launch(*cand)
                self.run(steps)
                t = self.run(steps)
            except _lib.DompapGPUError as exc:  # e.g. a CTA size this kernel cannot launch
                if verbose:
                    print(f"split_n={cand[0]:5d} threads_small={cand[1]:4d} threads_large={cand[2]:4d}: {exc}")
                continue
            if verbose:
                print(f"split_n={cand[0]:5d} threads_small={cand[1]:4d} threads_large={cand[2]:4d}: "
                      f"{t / steps:.4f} ms/step")
            if best is None or t < best[0]:
                best = (t, cand)
        if best is None:
            raise _lib.DompapGPUError("no launch shape of the candidates ran")
        self.set_launch(*best[1])
        return best[1], best[0] / steps

    # ---------------------------------------------------------------- results
    def state(self):
        """(positions, velocities, images) of all replicas, (N_total, D) each."""
        pos = np.empty((self.ntot, self.dim))
        vel = np.empty((self.ntot, self.dim))
        img = np.empty((self.ntot, self.dim), dtype=np.int32)
        _lib.check(_lib.load().dp_batch_get_state(self._h, _lib.dptr(pos), _lib.dptr(vel), _lib.iptr(img)))
        return pos, vel, img

    def replica_slice(self, r: int) -> slice:
        """Rows of replica ``r`` in the arrays of ``state()``."""
        return slice(int(self.offsets[r]), int(self.offsets[r + 1]))

    def last_forces(self) -> np.ndarray:
        """float32 pair forces of the last step of a ``run(..., record_forces=True)``."""
        out = np.empty((self.ntot, self.dim))
        _lib.check(_lib.load().dp_batch_last_forces(self._h, _lib.dptr(out)))
        return out

    def observables(self, reset: bool = True) -> dict:
        """Per-replica means over the sampled steps: potential energy per
        particle, temperature (sum m v^2 / (D N), as dompap's get_temperature)
        and pressure (W/V + sum m v^2 / (D V), as get_pressure)."""
        raw = np.empty((self.n_rep, 4))
        _lib.check(_lib.load().dp_batch_observables(self._h, _lib.dptr(raw), int(bool(reset))))
        ns = np.maximum(raw[:, 3], 1)
        n = self.counts.astype(np.float64)
        vol = np.prod(self.boxes, axis=1)
        u = raw[:, 0] / ns
        w = raw[:, 1] / ns
        mv2 = raw[:, 2] / ns
        return {"samples": raw[:, 3], "potential_energy_per_particle": u / n, "temperature": mv2 / (self.dim * n),
                "pressure": w / vol + mv2 / self.dim / vol, "virial": w}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                _lib.load().dp_batch_destroy(h)
            except Exception:
                pass
            self._h = None


def fcc_cells_for(n_target: int) -> tuple[int, int, int]:
    """Near-cubic fcc cells (a, b, c), each side k or k+1, with 4abc closest to n_target."""
    k = max(1, int(round((n_target / 4.0) ** (1.0 / 3.0))))
    best = None
    for a, b, c in itertools.product((k - 1, k, k + 1), repeat=3):
        if min(a, b, c) < 1 or max(a, b, c) - min(a, b, c) > 1:
            continue
        cand = (abs(4 * a * b * c - n_target), (a, b, c))
        if best is None or cand < best:
            best = cand
    return tuple(sorted(best[1], reverse=True))


def lj_replica_specs(n_rep: int = 4096, seed: int = 0, n_min: int = 64, n_max: int = 8192, t_min: float = 0.7,
                     t_max: float = 2.0, density: float = 0.8442, r_cut: float = 2.5, jitter: float = 0.02):
    """The batched LJ workload: N log-uniform in [n_min, n_max] rounded to an
    fcc count 4abc with near-cubic (a, b, c); T uniform in [t_min, t_max];
    fcc at ``density``; Maxwell-Boltzmann velocities. Draws whose box would be
    shorter than 2 r_cut are rejected and redrawn; returns (specs, rejected)."""
    rng = np.random.default_rng(seed)
    lat = (4.0 / density) ** (1.0 / 3.0)
    specs, rejected = [], 0
    while len(specs) < n_rep:
        n_draw = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        cells = fcc_cells_for(n_draw)
        box = np.array(cells, dtype=np.float64) * lat
        if box.min() < 2 * r_cut:
            rejected += 1
            continue
        pos = generate_positions(FCC, cells, (lat, lat, lat))
        pos = pos + rng.normal(0.0, jitter, size=pos.shape)
        pos = pos - np.floor(pos / box) * box
        temp = float(rng.uniform(t_min, t_max))
        vel = rng.normal(0.0, np.sqrt(temp), size=pos.shape)
        specs.append(ReplicaSpec(pos, vel, box, temp))
    return specs, rejected
