"""NumPy restatement of dompap's float64 hot path — TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use this
module, as the checker. Each function cites the reference ``file:line`` (paths
inside the dompap project) whose arithmetic it restates.

Exactness contract (pinned by ``tests/test_oracle_golden.py`` against fixtures
made by running the unmodified reference):

* pair sets (neighbour lists, including order and ``-1`` padding) are
  bit-identical: the same float64 subtraction, single-shift minimum image,
  sequential ``d0^2 + d1^2 + ...`` and IEEE ``sqrt`` compared ``< cutoff``;
* per-pair force / energy terms use the same operations in the same order;
* sums are sequential in the reference's loop order (``np.add.at`` and
  ``np.cumsum`` accumulate sequentially), so totals match the reference
  run under a sequential loop to the last bit.

sigma / epsilon are given either as Python floats (the reference's constant
lambdas, ``Simulation.py:513-524``) or as dense ``(N, N)`` float64 matrices
``sigma[n, m]`` (any index callable evaluated on all pairs, which is what the
reference's ``sigma_func(n, m)`` denotes).
"""
from __future__ import annotations

import numpy as np
import sympy as sp
from scipy.special import gamma

__all__ = [
    "make_pair_potential",
    "harmonic_repulsive",
    "generate_positions",
    "displacement",
    "neighbor_list_double_loop",
    "neighbor_counts",
    "neighbor_list_is_old",
    "forces_neighbor_list",
    "energy_neighbor_list",
    "virial_double_loop",
    "laplacian_neighbor_list",
    "forces_double_loop",
    "gjf_step",
    "leapfrog_step",
    "wrap_into_box",
    "radial_distribution_function",
    "pair_matrix",
]


# --------------------------------------------------------------------------
# pair potential  (dompap/potential.py:43-66, hard-coded form :10-40)
# --------------------------------------------------------------------------
def make_pair_potential(pair_potential_str: str = "(1-r)**2", r_cut: float = 1.0):
    """Return vectorised ``(u_cut, f_cut, c_cut)`` of the scaled distance.

    Restates ``dompap/potential.py:43-66``: ``f = -du/dr`` and ``c = d2u/dr2``
    by SymPy differentiation, lambdified to NumPy; ``u`` is shifted by
    ``u(r_cut)`` (:57-59); all three are 0 where ``r > r_cut`` (:61-65), so
    ``r == r_cut`` is kept. The force is NOT shifted.
    """
    r = sp.symbols("r")
    expr = sp.sympify(pair_potential_str)
    f_expr = sp.diff(-expr, r)
    c_expr = sp.diff(expr, r, 2)
    u_np = sp.lambdify(r, expr, "numpy")
    f_np = sp.lambdify(r, f_expr, "numpy")
    c_np = sp.lambdify(r, c_expr, "numpy")
    u_at_cut = u_np(np.float64(r_cut))

    def _bcast(fn, x):
        val = fn(x)
        return np.broadcast_to(np.asarray(val, dtype=np.float64), np.shape(x))

    def u_cut(x):
        x = np.asarray(x, dtype=np.float64)
        return np.where(x > r_cut, 0, _bcast(u_np, x) - u_at_cut)

    def f_cut(x):
        x = np.asarray(x, dtype=np.float64)
        return np.where(x > r_cut, 0, _bcast(f_np, x))

    def c_cut(x):
        x = np.asarray(x, dtype=np.float64)
        return np.where(x > r_cut, 0, _bcast(c_np, x))

    return u_cut, f_cut, c_cut


def harmonic_repulsive():
    """``'Harmonic repulsive'`` (dompap/potential.py:10-40): u = 0.5(1-r)^2,
    f = 1-r for r < 1, else 0; curvature 0; r_cut = 1."""

    def u(x):
        x = np.asarray(x, dtype=np.float64)
        return np.where(x < 1, 0.5 * (1 - x) ** 2, 0.0)

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        return np.where(x < 1, 1 - x, 0.0)

    def c(x):
        return np.zeros_like(np.asarray(x, dtype=np.float64))

    return u, f, c, 1.0


# --------------------------------------------------------------------------
# positions  (dompap/positions.py)
# --------------------------------------------------------------------------
def generate_positions(unit_cell_coordinates, cells, lattice_constants) -> np.ndarray:
    """Lattice from a unit cell (dompap/positions.py:33-52): cell index in
    C order (last axis fastest), basis particles consecutive, then scaled."""
    unit = np.asarray(unit_cell_coordinates, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int32)
    lat = np.asarray(lattice_constants, dtype=np.float64)
    n_cells = int(np.prod(cells))
    grid = np.stack(np.unravel_index(np.arange(n_cells), tuple(cells)), axis=1).astype(np.float64)
    pos = (grid[:, None, :] + unit[None, :, :]).reshape(n_cells * unit.shape[0], unit.shape[1])
    pos *= lat
    return pos


def _min_image(d: np.ndarray, box: np.ndarray) -> np.ndarray:
    """Single +-L shift per axis (dompap/positions.py:12-16)."""
    half = box / 2
    return np.where(d > half, d - box, np.where(d < -half, d + box, d))


def displacement(a: np.ndarray, b: np.ndarray, box: np.ndarray) -> np.ndarray:
    """``get_displacement_vector`` (dompap/positions.py:6-17), vectorised over rows."""
    return _min_image(np.asarray(a, np.float64) - np.asarray(b, np.float64), np.asarray(box, np.float64))


def _sq_sum(d: np.ndarray) -> np.ndarray:
    """Sequential ``d0^2 + d1^2 + ...`` over the last axis (NumPy/Numba sum of a short vector)."""
    acc = d[..., 0] * d[..., 0]
    for k in range(1, d.shape[-1]):
        acc = acc + d[..., k] * d[..., k]
    return acc


# --------------------------------------------------------------------------
# neighbour list  (dompap/neighbor_list.py)
# --------------------------------------------------------------------------
def neighbor_list_double_loop(positions, box_vectors, cutoff_distance, max_number_of_neighbors=None):
    """``get_neighbor_list_double_loop`` (dompap/neighbor_list.py:7-39).

    For each n, ascending m != n with ``sqrt(sum d^2) < cutoff`` (:25-33).
    Returns ``(nlist, counts)``; ``nlist`` is ``(N, K)`` int32, ``-1``-padded,
    ``K = max_number_of_neighbors`` (or the largest count when ``None``). The
    reference does not check overflow (:36-38); here rows longer than K are
    reported through ``counts`` (which holds the true neighbour counts).
    """
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_part = pos.shape[0]
    rows = []
    counts = np.zeros(n_part, dtype=np.int64)
    for n in range(n_part):
        d = _min_image(pos[n] - pos, box)
        dist = np.sqrt(_sq_sum(d))
        mask = dist < cutoff_distance
        mask[n] = False
        idx = np.nonzero(mask)[0]
        rows.append(idx)
        counts[n] = idx.size
    k = int(counts.max(initial=0)) if max_number_of_neighbors is None else int(max_number_of_neighbors)
    nl = np.full((n_part, k), -1, dtype=np.int32)
    for n, idx in enumerate(rows):
        m = min(idx.size, k)
        nl[n, :m] = idx[:m]
    return nl, counts


def neighbor_counts(neighbor_list: np.ndarray) -> np.ndarray:
    """``get_number_of_neighbors`` (dompap/neighbor_list.py:204-207)."""
    return np.sum(neighbor_list != -1, axis=1)


def neighbor_list_is_old(positions, old_positions, box_vectors, skin) -> bool:
    """``neighbor_list_is_old`` (dompap/neighbor_list.py:183-201): the largest
    min-image displacement^2 since the list was built vs ``(0.5 skin)^2``."""
    d = displacement(positions, old_positions, box_vectors)
    max_d2 = max(0.0, float(np.max(_sq_sum(d)))) if d.shape[0] else 0.0
    return max_d2 > (0.5 * skin) ** 2


# --------------------------------------------------------------------------
# pair sums  (dompap/potential.py)
# --------------------------------------------------------------------------
def pair_matrix(value, n_part: int) -> np.ndarray:
    """Dense ``(N, N)`` view of a sigma/epsilon specification (float or matrix)."""
    if np.isscalar(value):
        return np.full((n_part, n_part), float(value), dtype=np.float64)
    return np.asarray(value, dtype=np.float64)


def _pair_values(value, n_idx, m_idx):
    if np.isscalar(value):
        return np.float64(value)
    return np.asarray(value, dtype=np.float64)[n_idx, m_idx]


def _list_pairs(neighbor_list: np.ndarray):
    """(n, m) in the reference's loop order: row by row, stopping at the first -1
    (dompap/potential.py:177-179)."""
    nl = np.asarray(neighbor_list)
    valid = nl != -1
    # the reference breaks at the first -1 of a row
    first_pad = np.where(valid.all(axis=1), nl.shape[1], np.argmin(valid, axis=1))
    keep = np.arange(nl.shape[1])[None, :] < first_pad[:, None]
    n_idx, k_idx = np.nonzero(keep)
    return n_idx, nl[n_idx, k_idx].astype(np.int64)


def forces_neighbor_list(positions, box_vectors, pair_force, neighbor_list, sigma=1.0, epsilon=1.0):
    """``_get_forces`` (dompap/potential.py:163-188):
    ``F_n = sum_m eps * f(r/sigma) * d/r`` with d from the single-shift
    minimum image, ``r = (sum d^2) ** 0.5`` — no 1/sigma chain-rule factor."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_idx, m_idx = _list_pairs(neighbor_list)
    d = _min_image(pos[n_idx] - pos[m_idx], box)
    dist = _sq_sum(d) ** 0.5
    sig = _pair_values(sigma, n_idx, m_idx)
    eps = _pair_values(epsilon, n_idx, m_idx)
    scalar_force = eps * pair_force(dist / sig)
    unit = d / dist[:, None]
    forces = np.zeros_like(pos)
    np.add.at(forces, n_idx, scalar_force[:, None] * unit)
    return forces


def energy_neighbor_list(positions, box_vectors, pair_potential, neighbor_list, sigma=1.0, epsilon=1.0) -> float:
    """``_get_total_energy`` (dompap/potential.py:69-100): sequential
    ``sum eps * u(r/sigma)`` over the full list, halved."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_idx, m_idx = _list_pairs(neighbor_list)
    if n_idx.size == 0:
        return 0.0
    d = _min_image(pos[n_idx] - pos[m_idx], box)
    dist = np.sqrt(_sq_sum(d))
    sig = _pair_values(sigma, n_idx, m_idx)
    eps = _pair_values(epsilon, n_idx, m_idx)
    terms = eps * pair_potential(dist / sig).astype(np.float64)
    return float(np.cumsum(terms)[-1] / 2)


def pair_terms_abs_sum(positions, box_vectors, pair_fn, neighbor_list, sigma=1.0, epsilon=1.0) -> float:
    """``sum |eps * g(r/sigma)|`` over the list: the scale a summed quantity's
    rounding error is relative to (used to state tolerances)."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_idx, m_idx = _list_pairs(neighbor_list)
    d = _min_image(pos[n_idx] - pos[m_idx], box)
    dist = np.sqrt(_sq_sum(d))
    sig = _pair_values(sigma, n_idx, m_idx)
    eps = _pair_values(epsilon, n_idx, m_idx)
    return float(np.sum(np.abs(eps * pair_fn(dist / sig))))


def virial_double_loop(positions, box_vectors, pair_force, sigma=1.0, epsilon=1.0, return_abs=False):
    """``_get_virial_double_loop`` (dompap/potential.py:253-279):
    ``W = (1/D) sum_{n<m} eps f(r/sigma) r`` over ALL pairs, accumulated in
    the sequential ``for n: for m > n`` order."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_part, dim = pos.shape
    total = np.float64(0.0)
    abs_total = 0.0
    for n in range(n_part - 1):
        m_idx = np.arange(n + 1, n_part)
        d = _min_image(pos[n] - pos[m_idx], box)
        dist = _sq_sum(d) ** 0.5
        sig = _pair_values(sigma, np.full(m_idx.size, n), m_idx)
        eps = _pair_values(epsilon, np.full(m_idx.size, n), m_idx)
        w = eps * pair_force(dist / sig) * dist
        # sequential accumulation continuing from the running total
        acc = np.cumsum(np.concatenate(([total], w)))
        total = acc[-1]
        abs_total += float(np.sum(np.abs(w)))
    if return_abs:
        return float(total / dim), abs_total / dim
    return float(total / dim)


def laplacian_neighbor_list(positions, box_vectors, pair_force, pair_curvature, neighbor_list,
                            sigma=1.0, epsilon=1.0) -> np.ndarray:
    """``_get_laplacian`` (dompap/potential.py:327-364): per particle
    ``sum_m eps c(r/sigma) + (D-1) * (-eps f(r/sigma)) / r``."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    dim = pos.shape[1]
    n_idx, m_idx = _list_pairs(neighbor_list)
    d = _min_image(pos[n_idx] - pos[m_idx], box)
    d = _min_image(d, box)  # the reference applies the shift twice (:348-354)
    dist = _sq_sum(d) ** 0.5
    sig = _pair_values(sigma, n_idx, m_idx)
    eps = _pair_values(epsilon, n_idx, m_idx)
    scalar_force = eps * pair_force(dist / sig)
    dv_dr = -scalar_force
    d2v = eps * pair_curvature(dist / sig)
    terms = d2v + (dim - 1) * dv_dr / dist
    lap = np.zeros(pos.shape[0], dtype=np.float64)
    np.add.at(lap, n_idx, terms)
    return lap


def forces_double_loop(positions, box_vectors, pair_force, sigma=1.0, epsilon=1.0):
    """``_get_forces_double_loop`` (dompap/potential.py:217-250): all m != n,
    in ascending m, with ``f`` cut beyond r_cut by the potential itself."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_part = pos.shape[0]
    forces = np.zeros_like(pos)
    for n in range(n_part):
        m_idx = np.array([m for m in range(n_part) if m != n], dtype=np.int64)
        d = _min_image(pos[n] - pos[m_idx], box)
        dist = _sq_sum(d) ** 0.5
        sig = _pair_values(sigma, np.full(m_idx.size, n), m_idx)
        eps = _pair_values(epsilon, np.full(m_idx.size, n), m_idx)
        contrib = (eps * pair_force(dist / sig))[:, None] * (d / dist[:, None])
        acc = np.zeros(pos.shape[1])
        for c in contrib:
            acc = acc + c
        forces[n] = acc
    return forces


def forces_double_loop_single_core(positions, box_vectors, pair_force, sigma=1.0, epsilon=1.0):
    """``_get_forces_double_loop_single_core`` (dompap/potential.py:191-214):
    each pair n < m once, with sigma(n, m), epsilon(n, m), added to n and
    subtracted from m (Newton's third law), in the reference's loop order."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_part = pos.shape[0]
    forces = np.zeros_like(pos)
    for n in range(n_part - 1):
        m_idx = np.arange(n + 1, n_part, dtype=np.int64)
        d = _min_image(pos[n] - pos[m_idx], box)
        dist = np.sum(d ** 2, axis=1) ** 0.5
        sig = _pair_values(sigma, np.full(m_idx.size, n), m_idx)
        eps = _pair_values(epsilon, np.full(m_idx.size, n), m_idx)
        contrib = (eps * pair_force(dist / sig))[:, None] * (d / dist[:, None])
        for k, m in enumerate(m_idx):
            forces[n] = forces[n] + contrib[k]
            forces[m] = forces[m] - contrib[k]
    return forces


def energy_double_loop(positions, box_vectors, pair_potential, sigma=1.0, epsilon=1.0) -> float:
    """``_get_total_energy_double_loop`` (dompap/potential.py:103-130) and its
    single-core twin (:133-160): sum over n < m of eps(n, m) u(r/sigma(n, m)),
    not halved."""
    pos = np.asarray(positions, dtype=np.float64)
    box = np.asarray(box_vectors, dtype=np.float64)
    n_part = pos.shape[0]
    energy = 0.0
    for n in range(n_part - 1):
        m_idx = np.arange(n + 1, n_part, dtype=np.int64)
        d = _min_image(pos[n] - pos[m_idx], box)
        dist = np.sqrt(np.sum(d ** 2, axis=1))
        sig = _pair_values(sigma, np.full(m_idx.size, n), m_idx)
        eps = _pair_values(epsilon, np.full(m_idx.size, n), m_idx)
        for t in eps * pair_potential(dist / sig).astype(np.float64):
            energy = energy + t
    return float(energy)


# --------------------------------------------------------------------------
# integrators  (dompap/integrator.py)
# --------------------------------------------------------------------------
def gjf_step(positions, velocities, betas, forces, masses, time_step, temperature_target,
             temperature_damping_time, normals):
    """``make_one_step`` (dompap/integrator.py:17-40), the G-JF leap-frog
    (arXiv:1303.7011 Sec. II.C, eqs. 16-17), with the standard normal deviates
    passed in (the reference draws them with ``np.random.normal`` at :30)."""
    masses = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    alphas = masses / temperature_damping_time
    beta_variance = 2 * alphas * temperature_target * time_step
    new_betas = np.sqrt(beta_variance) * normals
    numerator = 1.0 - alphas * time_step / 2.0 / masses
    denominator = 1.0 + alphas * time_step / 2.0 / masses
    a = numerator / denominator
    b = 1 / denominator
    velocities = a * velocities + b * time_step * forces / masses + b * (betas + new_betas) / 2 / masses
    positions = positions + velocities * time_step
    return positions, velocities, new_betas


def leapfrog_step(positions, velocities, forces, masses, time_step):
    """``make_one_step_leap_frog`` (dompap/integrator.py:5-14)."""
    masses = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    velocities = velocities + time_step * forces / masses
    positions = positions + time_step * velocities
    return positions, velocities


def wrap_into_box(positions, image_positions, box_vectors):
    """``wrap_into_box`` (dompap/positions.py:90-98), in place."""
    shift = np.floor(positions / box_vectors[np.newaxis, :], dtype=np.float64)
    image_positions += shift.astype(np.int32)
    positions -= shift * box_vectors[np.newaxis, :]


# --------------------------------------------------------------------------
# observables
# --------------------------------------------------------------------------
def radial_distribution_function(positions_n, positions_m, box_vectors, r_bins):
    """``get_radial_distribution_function`` (dompap/positions.py:58-87):
    ``np.round`` minimum image, histogram of all N_n*N_m distances (self
    pairs included), normalised by the pair count and the D-sphere shell."""
    r_bins = np.asarray(r_bins, dtype=np.float64)
    if not np.all(np.diff(r_bins) >= 0):
        raise ValueError("r_bins array must be sorted in ascending order.")
    box_vectors = np.asarray(box_vectors, dtype=np.float64)
    diff = positions_n[:, np.newaxis, :] - positions_m[np.newaxis, :, :]
    for i in range(diff.shape[-1]):
        box_length = np.linalg.norm(box_vectors[i])
        diff[:, :, i] -= box_length * np.round(diff[:, :, i] / box_length)
    distances = np.linalg.norm(diff, axis=2)
    histogram = np.histogram(distances, bins=r_bins)[0]
    number_of_pairs = positions_n.shape[0] * positions_m.shape[0]
    box_volume = np.prod(box_vectors)
    dr_bins = np.diff(r_bins)
    r_mid = r_bins[:-1] + dr_bins / 2
    dims = positions_n.shape[1]
    surface = 2 * np.pi ** (dims / 2) / gamma(dims / 2)
    shell_volume = surface * r_mid ** (dims - 1) * dr_bins
    return r_mid, histogram / shell_volume / number_of_pairs * box_volume


# --------------------------------------------------------------------------
# the Simulation step loop  (dompap/Simulation.py:681-737)
# --------------------------------------------------------------------------
class OracleSystem:
    """Minimal restatement of ``Simulation``'s per-step sequence
    (dompap/Simulation.py:681-724): skin check -> (rebuild) -> forces ->
    integrate -> wrap, with the double-loop neighbour list."""

    def __init__(self, positions, velocities, masses, box, pair_potential_str, r_cut, skin,
                 sigma=1.0, epsilon=1.0, max_neighbors=512, hardcoded=False):
        self.positions = np.array(positions, dtype=np.float64)
        self.velocities = np.array(velocities, dtype=np.float64)
        self.betas = np.zeros_like(self.positions)
        self.images = np.zeros(self.positions.shape, dtype=np.int32)
        self.masses = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
        self.box = np.asarray(box, dtype=np.float64)
        if hardcoded:
            self.u, self.f, self.c, self.r_cut = harmonic_repulsive()
        else:
            self.u, self.f, self.c = make_pair_potential(pair_potential_str, r_cut)
            self.r_cut = r_cut
        self.skin = skin
        self.sigma, self.epsilon = sigma, epsilon
        self.kmax = max_neighbors
        self.rebuilds = 0
        self.set_neighbor_list()

    def largest_sigma(self):
        # dompap/Simulation.py:346-351 scans sigma_func over all (n, m)
        return float(np.max(pair_matrix(self.sigma, self.positions.shape[0])))

    def set_neighbor_list(self):
        cutoff = self.largest_sigma() * self.r_cut + self.skin
        self.nlist, self.counts = neighbor_list_double_loop(self.positions, self.box, cutoff, self.kmax)
        self.reference_positions = self.positions.copy()
        self.rebuilds += 1

    def update_neighbor_list(self):
        if neighbor_list_is_old(self.positions, self.reference_positions, self.box, self.skin):
            self.set_neighbor_list()

    def forces(self):
        self.update_neighbor_list()
        return forces_neighbor_list(self.positions, self.box, self.f, self.nlist, self.sigma, self.epsilon)

    def step_leap_frog(self):
        self.update_neighbor_list()
        f = self.forces()
        self.positions, self.velocities = leapfrog_step(self.positions, self.velocities, f, self.masses, self.dt)
        wrap_into_box(self.positions, self.images, self.box)

    def step_gjf(self, normals):
        self.update_neighbor_list()
        f = self.forces()
        self.positions, self.velocities, self.betas = gjf_step(
            self.positions, self.velocities, self.betas, f, self.masses, self.dt, self.temperature,
            self.damping_time, normals)
        wrap_into_box(self.positions, self.images, self.box)

    dt = 0.01
    temperature = 1.0
    damping_time = 0.1
