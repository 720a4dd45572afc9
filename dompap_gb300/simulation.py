"""Drop-in ``Simulation`` for dompap's (dompap/Simulation.py) with every
per-step operation on the GPU.

The class keeps dompap's fields, method names, arguments, defaults, dispatch
strings and errors. Host NumPy arrays are mirrors of the device state:

* after ``run``/``step`` the device holds the newest positions, velocities,
  betas and images; reading one of these attributes downloads it;
* an attribute that was read (or assigned) may have been modified in place by
  the caller, so it is uploaded again before the next GPU operation
  (dirty-on-read), which keeps in-place edits such as
  ``sim.positions[0] = [...]`` working as in dompap.

``run`` never copies state back to the host.

sigma/epsilon are floats, ``(ntypes, ntypes)`` arrays indexed by
``particle_types`` (an extension), or index callables ``f(n, m)``. A callable
is evaluated on all pairs (vectorised when it accepts index arrays) and is
turned into a per-type table when it factors through ``particle_types``,
otherwise into a dense ``(N, N)`` matrix (N <= 8192).

The method strings keep dompap's meanings for the pair set. ``'double loop'``
(dompap's default) builds the list by an all-pairs pass in ascending index
order for N <= 16384 and by the exact cell-list pass above that; both give
the same pair set as dompap's double loop. ``'cell list'`` always uses the
cell-list pass (exact, unlike dompap/neighbor_list.py:106-180).
"""
from __future__ import annotations

import os
from copy import deepcopy

import numpy as np

from . import _lib
from . import codegen
from .positions import generate_positions

DEFAULT_SPATIAL_DIMENSION = 3
DEFAULT_NUMBER_OF_PARTICLES = 125
_ALLPAIRS_LIMIT = 16384
_DENSE_LIMIT = 8192

# dompap's force / energy method strings -> the GPU kernels
_FORCE_METHOD_CODES = {"neighbor list": _lib.DP_METHOD_LIST, "double loop": _lib.DP_METHOD_ALLPAIRS,
                       "vectorized": _lib.DP_METHOD_ALLPAIRS,
                       "double loop single core": _lib.DP_METHOD_ALLPAIRS_NEWTON}
_ENERGY_METHOD_CODES = {"neighbor list": _lib.DP_METHOD_LIST, "double loop": _lib.DP_METHOD_ALLPAIRS,
                        "double loop single core": _lib.DP_METHOD_ALLPAIRS}

_STATE = ("positions", "velocities", "betas", "image_positions")
_HOST_ONLY = ("masses", "particle_types", "box_vectors")


def _default_positions():
    pos = np.zeros((DEFAULT_NUMBER_OF_PARTICLES, DEFAULT_SPATIAL_DIMENSION), dtype=np.float64)
    for i in range(5):
        for j in range(5):
            for k in range(5):
                pos[i * 25 + j * 5 + k] = [i, j, k]
    return pos


def _const_func(value):
    v = np.float64(value)
    return lambda n, m: v


class Simulation:
    """GPU drop-in for ``dompap.Simulation`` (dompap/Simulation.py:67-1229).

    The default system is dompap's: a 5x5x5 simple-cubic lattice of unit-mass
    particles in a 5x5x5 box, the harmonic repulsive pair potential (1-r)**2
    truncated at r_cut = 1, neighbour-list skin 1.0, the Langevin G-JF
    integrator with time step 0.01, target temperature 1.0 and damping time 0.1.
    """

    energy_method_str = "neighbor list"
    force_method_str = "neighbor list"
    neighbor_list_method_str = "double loop"
    _KNOWN_ENERGY_METHODS = {"neighbor list", "double loop", "double loop single core"}
    _KNOWN_FORCE_METHODS = {"neighbor list", "double loop", "double loop single core", "vectorized"}
    _KNOWN_CELL_LIST_METHODS = {"cell list", "double loop"}
    _KNOWN_PRECISIONS = {"fp64": _lib.DP_PREC_FP64, "fp32": _lib.DP_PREC_FP32, "mlp": _lib.DP_PREC_MLP}

    def __init__(self, particle_types=None, positions=None, box_vectors=None, image_positions=None,
                 velocities=None, betas=None, neighbor_list=None, positions_neighbour_list=None, masses=None,
                 pair_potential_r_cut=np.float64(1.0), neighbor_list_skin=np.float64(1.0),
                 max_number_of_neighbors=np.int32(512), number_of_neighbor_list_updates=0, number_of_steps=0,
                 time_step=np.float64(0.01), temperature_target=np.float64(1.0),
                 temperature_damping_time=np.float64(0.1), pair_potential=None, pair_potential_str=None,
                 pair_force=None, pair_curvature=None, epsilon_func=None, sigma_func=None, precision="fp64"):
        d = self.__dict__
        d["_h"] = None
        d["_dev_newer"] = set()
        d["_host_dirty"] = set()
        d["_precision"] = self._KNOWN_PRECISIONS[precision]
        n = DEFAULT_NUMBER_OF_PARTICLES
        d["_particle_types"] = (np.zeros((n, 1), dtype=np.int32) if particle_types is None
                                else np.asarray(particle_types, dtype=np.int32).reshape(-1, 1))
        d["_positions"] = _default_positions() if positions is None else np.array(positions, dtype=np.float64)
        d["_box_vectors"] = (np.array([5, 5, 5], dtype=np.float64) if box_vectors is None
                             else np.array(box_vectors, dtype=np.float64))
        shape = d["_positions"].shape
        d["_image_positions"] = (np.zeros(shape, dtype=np.int32) if image_positions is None
                                 else np.array(image_positions, dtype=np.int32))
        d["_velocities"] = (np.random.normal(loc=0.0, scale=1.0, size=shape) if velocities is None
                            else np.array(velocities, dtype=np.float64))
        d["_betas"] = np.zeros(shape, dtype=np.float64) if betas is None else np.array(betas, dtype=np.float64)
        d["_masses"] = (np.ones((shape[0], 1), dtype=np.float64) if masses is None
                        else np.asarray(masses, dtype=np.float64).reshape(-1, 1))
        self.pair_potential_r_cut = np.float64(pair_potential_r_cut)
        self.neighbor_list_skin = np.float64(neighbor_list_skin)
        self.max_number_of_neighbors = np.int32(max_number_of_neighbors)
        d["_nl_count_base"] = int(number_of_neighbor_list_updates)
        d["_dev_rebuilds_base"] = 0
        self.number_of_steps = int(number_of_steps)
        self.time_step = np.float64(time_step)
        self.temperature_target = np.float64(temperature_target)
        self.temperature_damping_time = np.float64(temperature_damping_time)
        self.pair_potential_str = pair_potential_str
        self.epsilon_func = epsilon_func if epsilon_func is not None else _const_func(1.0)
        self.sigma_func = sigma_func if sigma_func is not None else _const_func(1.0)
        d["_sigma_spec"] = 1.0
        d["_epsilon_spec"] = 1.0
        d["_pot_source"] = None
        d["_surrogate"] = None
        d["_seed"] = int(np.random.randint(0, 2**62, dtype=np.int64))
        # dompap/Simulation.py:149-153
        self.set_pair_potential()
        self.set_pair_potential_parameters(sigma=1.0, epsilon=1.0)
        self.set_neighbor_list()

    # ------------------------------------------------------------------ mirrors
    def _pull(self, name):
        if name in self._dev_newer and self._h is not None:
            arr = self.__dict__["_" + name]
            h = self._h
            if name == "positions":
                _lib.check(_lib.load().dp_get_positions(h, _lib.dptr(arr)))
            elif name == "velocities":
                _lib.check(_lib.load().dp_get_velocities(h, _lib.dptr(arr)))
            elif name == "betas":
                _lib.check(_lib.load().dp_get_betas(h, _lib.dptr(arr)))
            elif name == "image_positions":
                _lib.check(_lib.load().dp_get_images(h, _lib.iptr(arr)))
            self._dev_newer.discard(name)

    def __getattr__(self, name):
        # only called when normal lookup fails: the mirrored arrays
        if name in _STATE or name in _HOST_ONLY:
            d = self.__dict__
            if name in _STATE:
                self._pull(name)
            d["_host_dirty"].add(name)
            return d["_" + name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _STATE or name in _HOST_ONLY:
            d = self.__dict__
            # always a private copy: device results are written into it in place
            if name in ("image_positions", "particle_types"):
                value = np.array(value, dtype=np.int32, order="C")
            else:
                value = np.array(value, dtype=np.float64, order="C")
            d["_" + name] = value
            d["_dev_newer"].discard(name)
            d["_host_dirty"].add(name)
            return
        if name in ("neighbor_list", "positions_neighbour_list"):
            raise AttributeError(f"{name} is computed on the GPU and read-only")
        object.__setattr__(self, name, value)

    @property
    def number_of_neighbor_list_updates(self) -> int:
        if self._h is None:
            return self._nl_count_base
        st = self._stats()
        return self._nl_count_base + int(st.rebuilds) - self._dev_rebuilds_base

    @number_of_neighbor_list_updates.setter
    def number_of_neighbor_list_updates(self, value):
        self.__dict__["_nl_count_base"] = int(value)
        self.__dict__["_dev_rebuilds_base"] = int(self._stats().rebuilds) if self._h is not None else 0

    # ------------------------------------------------------------------ device
    def _lib(self):
        return _lib.load()

    def _ensure_handle(self):
        """Create (or re-create on a shape change) the device system and upload it."""
        d = self.__dict__
        pos = d["_positions"]
        n, dim = pos.shape
        if d.get("_h_shape") == (n, dim) and d["_h"] is not None:
            return
        lib = self._lib()
        rebuilds = 0
        if d["_h"] is not None:
            rebuilds = int(self._stats().rebuilds) - d["_dev_rebuilds_base"]
            lib.dp_destroy(d["_h"])
            d["_h"] = None
        h = _lib.ctypes.c_void_p()
        create_prec = _lib.DP_PREC_FP32 if d["_precision"] == _lib.DP_PREC_MLP else d["_precision"]
        _lib.check(lib.dp_create(dim, n, create_prec, _lib.ctypes.byref(h)))
        d["_h"] = h
        d["_h_shape"] = (n, dim)
        d["_methods_uploaded"] = None
        lanes, blocks = d.get("_step_launch", (0, 0))
        if lanes or blocks:
            _lib.check(lib.dp_set_step_launch(h, int(lanes), int(blocks)))
        d["_nl_count_base"] += rebuilds
        d["_dev_rebuilds_base"] = 0
        d["_dev_newer"].clear()
        d["_host_dirty"].update(_STATE + _HOST_ONLY)
        d["_params_dirty"] = True
        d["_pot_dirty"] = True
        d["_nl_dirty"] = True
        d["_int_dirty"] = True

    def _push(self):
        """Upload host-side changes before a GPU operation."""
        self._ensure_handle()
        d = self.__dict__
        lib = self._lib()
        h = d["_h"]
        dirty = d["_host_dirty"]
        n, dim = d["_positions"].shape
        if "box_vectors" in dirty:
            box = np.ascontiguousarray(d["_box_vectors"], dtype=np.float64)
            if box.shape != (dim,):
                raise ValueError(f"box_vectors must have shape ({dim},), got {box.shape}")
            _lib.check(lib.dp_set_box(h, _lib.dptr(box)))
            if box.tobytes() != d.get("_box_uploaded", b""):
                d["_box_uploaded"] = box.tobytes()
                d["_nl_dirty"] = True
        for name, fn in (("positions", lib.dp_set_positions), ("velocities", lib.dp_set_velocities),
                         ("betas", lib.dp_set_betas)):
            if name in dirty:
                arr = np.ascontiguousarray(d["_" + name], dtype=np.float64)
                if arr.shape != (n, dim):
                    raise ValueError(f"{name} must have shape {(n, dim)}, got {arr.shape}")
                _lib.check(fn(h, _lib.dptr(arr)))
        if "image_positions" in dirty:
            arr = np.ascontiguousarray(d["_image_positions"], dtype=np.int32)
            if arr.shape != (n, dim):
                raise ValueError(f"image_positions must have shape {(n, dim)}, got {arr.shape}")
            _lib.check(lib.dp_set_images(h, _lib.iptr(arr)))
        keep = set()
        if "masses" in dirty:
            m = np.ascontiguousarray(np.asarray(d["_masses"], dtype=np.float64).reshape(-1))
            if m.shape == (n,):
                _lib.check(lib.dp_set_masses(h, _lib.dptr(m)))
                d["_int_dirty"] = True
            else:
                keep.add("masses")  # stale after a shape change, as in dompap; checked by _require_masses
        if "particle_types" in dirty:
            t = np.ascontiguousarray(np.asarray(d["_particle_types"], dtype=np.int32).reshape(-1))
            if t.shape == (n,):
                _lib.check(lib.dp_set_types(h, _lib.iptr(t)))
                d["_params_dirty"] = True
            else:
                keep.add("particle_types")
        dirty.clear()
        dirty.update(keep)
        if d.get("_pot_dirty"):
            sur = d.get("_surrogate")
            if d["_precision"] == _lib.DP_PREC_MLP and sur is not None:
                src, _ = sur.cheap_source()
                _lib.check(lib.dp_set_mlp(h, sur._h))
            else:
                src = d["_pot_source"]
            _lib.check(lib.dp_set_potential(h, src.encode(), float(self.pair_potential_r_cut)))
            if d["_precision"] == _lib.DP_PREC_MLP:
                _lib.check(lib.dp_set_precision(h, _lib.DP_PREC_MLP))
            d["_pot_dirty"] = False
            d["_nl_dirty"] = True
        if d.get("_params_dirty"):
            self._upload_pair_params()
            d["_params_dirty"] = False
            d["_nl_dirty"] = True
        if d.get("_int_dirty"):
            _lib.check(lib.dp_set_integrator(h, float(self.time_step), float(self.temperature_target),
                                             float(self.temperature_damping_time), d["_seed"] & (2**64 - 1)))
            d["_int_dirty"] = False
        methods = self._pair_method_codes()
        if d.get("_methods_uploaded") != methods:
            _lib.check(lib.dp_set_pair_methods(h, *methods))
            d["_methods_uploaded"] = methods
        if d.get("_nl_dirty"):
            method = self._nl_method_code()
            _lib.check(lib.dp_set_neighbor_list(h, float(self.neighbor_list_skin),
                                                int(self.max_number_of_neighbors), method))
            d["_nl_dirty"] = False

    def _pair_method_codes(self):
        """dompap's force and energy method strings -> the GPU kernels
        (neighbour-list kernels, or the all-pairs kernels for the double-loop
        and vectorised methods, dompap/potential.py:103-160,191-250,298-324)."""
        return (_FORCE_METHOD_CODES.get(self.force_method_str, _lib.DP_METHOD_LIST),
                _ENERGY_METHOD_CODES.get(self.energy_method_str, _lib.DP_METHOD_LIST))

    def _nl_method_code(self):
        n = self.__dict__["_positions"].shape[0]
        if self.neighbor_list_method_str == "double loop" and n <= _ALLPAIRS_LIMIT:
            return _lib.DP_NL_ALLPAIRS
        return _lib.DP_NL_CELL

    def _require_masses(self):
        d = self.__dict__
        n = d["_positions"].shape[0]
        if d["_masses"].shape != (n, 1):
            raise ValueError(f"Expected shape of masses: {(n, 1)}, got: {d['_masses'].shape}")

    def _stats(self) -> _lib.DpStats:
        st = _lib.DpStats()
        _lib.check(self._lib().dp_get_stats(self._h, _lib.ctypes.byref(st)))
        return st

    def _mark_device_newer(self):
        self._dev_newer.update(_STATE)
        for name in _STATE:
            self._host_dirty.discard(name)

    # ------------------------------------------------------------ pair params
    def _pair_table(self, spec, name):
        """float | (T,T) array | callable -> (mode, ntypes, flat table)."""
        n = self.__dict__["_positions"].shape[0]
        types = np.asarray(self.__dict__["_particle_types"], dtype=np.int64).reshape(-1)
        if isinstance(spec, (float, int, np.floating, np.integer)):
            return _lib.DP_PAIR_CONST, 1, np.array([float(spec)])
        if isinstance(spec, np.ndarray) and spec.ndim == 2 and spec.shape[0] == spec.shape[1] and spec.shape[0] != n:
            return _lib.DP_PAIR_TYPES, spec.shape[0], np.ascontiguousarray(spec, dtype=np.float64).reshape(-1)
        if isinstance(spec, np.ndarray) and spec.shape == (n, n):
            mat = np.ascontiguousarray(spec, dtype=np.float64)
        elif callable(spec):
            mat = self._evaluate_pair_callable(spec, n)
        else:
            raise ValueError(f"Unknown type of {name}: {type(spec)}")
        # a matrix that factors through particle_types becomes a type table
        if types.shape == (n,) and n <= 4096 and types.min(initial=0) >= 0 and types.max(initial=0) < 64:
            nt = int(types.max(initial=0)) + 1
            off = ~np.eye(n, dtype=bool)
            ti = np.broadcast_to(types[:, None], (n, n))[off]
            tj = np.broadcast_to(types[None, :], (n, n))[off]
            table = np.ones((nt, nt))
            table[ti, tj] = mat[off]
            if np.array_equal(table[ti, tj], mat[off]):
                return _lib.DP_PAIR_TYPES, nt, np.ascontiguousarray(table).reshape(-1)
        return _lib.DP_PAIR_DENSE, 1, mat.reshape(-1)

    @staticmethod
    def _evaluate_pair_callable(fn, n):
        if n > _DENSE_LIMIT:
            raise ValueError(
                f"sigma/epsilon callables are evaluated on all N^2 pairs, which is limited to N <= {_DENSE_LIMIT}; "
                "for larger systems pass an (ntypes, ntypes) array with set_types()")
        idx = np.arange(n)
        try:
            with np.errstate(all="ignore"):
                mat = np.asarray(fn(idx[:, None], idx[None, :]), dtype=np.float64)
            if mat.shape == (n, n):
                return np.ascontiguousarray(mat)
        except Exception:  # not vectorisable: evaluate pair by pair
            pass
        mat = np.empty((n, n), dtype=np.float64)
        for a in range(n):
            for b in range(n):
                mat[a, b] = fn(a, b)
        return mat

    def _upload_pair_params(self):
        d = self.__dict__
        ms, ns, st = self._pair_table(d["_sigma_spec"], "sigma")
        me, ne, et = self._pair_table(d["_epsilon_spec"], "epsilon")
        if ms != me or ns != ne:
            # bring both to the more general representation
            n = d["_positions"].shape[0]
            mode = max(ms, me)
            if mode == _lib.DP_PAIR_TYPES:
                nt = max(ns, ne)
                st = self._expand_types(ms, st, nt)
                et = self._expand_types(me, et, nt)
                ns = ne = nt
            else:
                st = self._dense(ms, st, ns, n)
                et = self._dense(me, et, ne, n)
                ns = ne = 1
            ms = me = mode
        st = np.ascontiguousarray(st, dtype=np.float64)
        et = np.ascontiguousarray(et, dtype=np.float64)
        _lib.check(self._lib().dp_set_pair_params(d["_h"], ms, ns, _lib.dptr(st), _lib.dptr(et)))

    @staticmethod
    def _expand_types(mode, table, nt):
        if mode == _lib.DP_PAIR_CONST:
            return np.full(nt * nt, table[0])
        t = table.reshape(int(np.sqrt(table.size)), -1)
        out = np.ones((nt, nt))
        out[: t.shape[0], : t.shape[1]] = t
        return out.reshape(-1)

    def _dense(self, mode, table, nt, n):
        if mode == _lib.DP_PAIR_CONST:
            return np.full(n * n, table[0])
        if mode == _lib.DP_PAIR_TYPES:
            types = np.asarray(self.__dict__["_particle_types"], dtype=np.int64).reshape(-1)
            t = table.reshape(nt, nt)
            return t[types[:, None], types[None, :]].reshape(-1)
        return table

    # ------------------------------------------------------------------ API
    def __str__(self):
        pos = self.__getattr__("positions")
        masses = self.__getattr__("masses")
        return f"""Simulation:
    positions: {pos[:1]} ... {pos[-1:]}
    box_vectors: {self.__getattr__('box_vectors')}
    masses: {masses[:1]} ... {masses[-1:]}"""

    def copy(self):
        """Deep copy with its own device system (dompap/Simulation.py:162-187)."""
        return deepcopy(self)

    def __deepcopy__(self, memo):
        for name in _STATE:
            self._pull(name)
        new = object.__new__(type(self))
        nd = new.__dict__
        for k, v in self.__dict__.items():
            if k in ("_h", "_h_shape"):
                continue
            shared = ("sigma_func", "epsilon_func", "_sigma_spec", "_epsilon_spec", "_surrogate")
            nd[k] = deepcopy(v, memo) if k not in shared else v
        nd["_h"] = None
        nd["_dev_newer"] = set()
        nd["_host_dirty"] = set()
        nd["_seed"] = int(np.random.randint(0, 2**62, dtype=np.int64))
        nd["_nl_count_base"] = self.number_of_neighbor_list_updates
        nd["_dev_rebuilds_base"] = 0
        new._push()
        # the copy's list is built from the same positions
        _lib.check(new._lib().dp_update_neighbor_list(new._h, 0, None))
        nd["_dev_rebuilds_base"] = int(new._stats().rebuilds)
        return new

    def set_positions(self, unit_cell_coordinates=([0.0, 0.0, 0.0],), cells=(5, 5, 5),
                      lattice_constants=(1.0, 1.0, 1.0)):
        """Lattice positions (dompap/Simulation.py:189-230)."""
        unit = np.array(unit_cell_coordinates, dtype=np.float64)
        cells = np.array(cells, dtype=np.int32)
        lat = np.array(lattice_constants, dtype=np.float64)
        self.box_vectors = np.array(cells, dtype=np.float64) * np.array(lat, dtype=np.float64)
        positions = generate_positions(unit, cells, lat)
        self.positions = positions
        self.image_positions = np.zeros(positions.shape, dtype=np.int32)
        d = self.__dict__
        if d["_betas"].shape != positions.shape:
            self.betas = np.zeros(positions.shape, dtype=np.float64)
        if d["_velocities"].shape != positions.shape:
            self.velocities = np.random.normal(loc=0.0, scale=1.0, size=positions.shape).astype(np.float64)

    def set_masses(self, masses: float | list | np.ndarray = 1.0):
        """dompap/Simulation.py:232-276."""
        n = self.__dict__["_positions"].shape[0]
        if isinstance(masses, float) or isinstance(masses, int):
            new = np.ones((n, 1), dtype=np.float64) * np.float64(masses)
        elif isinstance(masses, list):
            new = np.array(masses, dtype=np.float64).reshape(-1, 1)
        elif isinstance(masses, np.ndarray):
            new = masses.reshape(-1, 1)
        else:
            raise ValueError(f"Unknown type of masses: {type(masses)}")
        expected_shape = (n, 1)
        if new.shape != expected_shape:
            raise ValueError(f"Expected shape of masses: {expected_shape}, got: {new.shape}")
        self.masses = new
        if self.__dict__["_masses"].shape != self.__dict__["_particle_types"].shape:
            self.particle_types = np.zeros(self.__dict__["_masses"].shape, dtype=np.int32)

    def set_random_velocities(self, temperature: float = 1.0):
        """Normal velocities with variance T/m (dompap/Simulation.py:278-290)."""
        d = self.__dict__
        self.velocities = np.random.normal(loc=0.0, scale=np.sqrt(temperature / d["_masses"]),
                                           size=d["_positions"].shape).astype(np.float64)

    def set_types(self, types: int | list = 0):
        """dompap/Simulation.py:292-305."""
        n = self.__dict__["_positions"].shape[0]
        if isinstance(types, int):
            new = np.ones((n, 1), dtype=np.int32) * np.int32(types)
        elif isinstance(types, list):
            new = np.array(types, dtype=np.int32).reshape(-1, 1)
        elif isinstance(types, np.ndarray):
            new = types.astype(np.int32).reshape(-1, 1)
        else:
            raise ValueError(f"Unknown type of types: {type(types)}")
        expected_shape = (n, 1)
        if new.shape != expected_shape:
            raise ValueError(f"Expected shape of types is {expected_shape} but got {new.shape}")
        self.particle_types = new

    def set_particle_types(self, types) -> None:
        """dompap/Simulation.py:1003-1017."""
        self.particle_types = np.ones_like(self.__dict__["_masses"], dtype=np.int32) * types

    def set_neighbor_list(self, skin: float = None, max_number_of_neighbors: int = None,
                          method_str: None | str = None) -> None:
        """Rebuild the neighbour list now (dompap/Simulation.py:307-381)."""
        if skin is not None:
            self.neighbor_list_skin = np.float64(skin)
        if max_number_of_neighbors is not None:
            self.max_number_of_neighbors = np.int32(max_number_of_neighbors)
        if method_str is not None:
            if method_str not in self._KNOWN_CELL_LIST_METHODS:
                raise ValueError(
                    f"Unknown neighbor list method: {method_str}. Try: {self._KNOWN_CELL_LIST_METHODS}.")
            self.neighbor_list_method_str = method_str
        if self.neighbor_list_method_str not in self._KNOWN_CELL_LIST_METHODS:
            raise ValueError(f"Unknown neighbor list method: {self.neighbor_list_method_str}")
        self.__dict__["_nl_dirty"] = True
        self._push()
        _lib.check(self._lib().dp_update_neighbor_list(self._h, 0, None))

    def update_neighbor_list(self, check=True) -> None:
        """Rebuild if a particle moved more than skin/2 (dompap/Simulation.py:383-401)."""
        self._push()
        _lib.check(self._lib().dp_update_neighbor_list(self._h, 1 if check else 0, None))

    @property
    def neighbor_list(self) -> np.ndarray:
        """(N, max_number_of_neighbors) int32, rows ascending, -1 padded."""
        self._push()
        n = self.__dict__["_positions"].shape[0]
        k = int(self.max_number_of_neighbors)
        out = np.empty((n, k), dtype=np.int32)
        mc = _lib.ctypes.c_int32(0)
        _lib.check(self._lib().dp_get_neighbor_list(self._h, _lib.iptr(out), k, _lib.ctypes.byref(mc)))
        return out

    @property
    def positions_neighbour_list(self) -> np.ndarray:
        self._push()
        out = np.empty(self.__dict__["_positions"].shape, dtype=np.float64)
        _lib.check(self._lib().dp_get_reference_positions(self._h, _lib.dptr(out)))
        return out

    def set_pair_potential(self, pair_potential_str: str = "(1-r)**2", r_cut: float = 1.0, force_method=None,
                           energy_method=None) -> None:
        """SymPy string -> CUDA (NVRTC) pair potential (dompap/Simulation.py:403-467)."""
        src, rc = codegen.make_pair_source(pair_potential_str, r_cut)
        if pair_potential_str in codegen.HARDCODED:
            self.pair_potential_str = codegen.HARDCODED[pair_potential_str][0]
        else:
            self.pair_potential_str = pair_potential_str
        self.pair_potential_r_cut = np.float64(rc)
        d = self.__dict__
        d["_pot_source"] = src
        d["_pot_dirty"] = True
        if pair_potential_str not in codegen.HARDCODED:
            if force_method is not None:
                if force_method not in self._KNOWN_FORCE_METHODS:
                    raise ValueError(f"Unknown force method: {force_method}. Try: {self._KNOWN_FORCE_METHODS}.")
                self.force_method_str = force_method
            if energy_method is not None:
                if energy_method not in self._KNOWN_ENERGY_METHODS:
                    raise ValueError(
                        f"Unknown energy method: {energy_method}. Try: {self._KNOWN_ENERGY_METHODS}.")
                self.energy_method_str = energy_method
        self.set_neighbor_list()

    @property
    def pair_potential(self):
        return self._pair_callable(0)

    @property
    def pair_force(self):
        return self._pair_callable(1)

    @property
    def pair_curvature(self):
        return self._pair_callable(2)

    def _pair_callable(self, which):
        def fn(r):
            self._push()
            arr = np.ascontiguousarray(np.asarray(r, dtype=np.float64).reshape(-1))
            u = np.empty_like(arr)
            f = np.empty_like(arr)
            c = np.empty_like(arr)
            _lib.check(self._lib().dp_eval_potential(self._h, _lib.dptr(arr), arr.size, _lib.dptr(u),
                                                     _lib.dptr(f), _lib.dptr(c)))
            out = (u, f, c)[which].reshape(np.shape(r))
            return out[()] if out.ndim == 0 else out

        return fn

    def set_pair_potential_parameters(self, sigma: float = 1.0, epsilon: float = 1.0) -> None:
        """sigma/epsilon as floats, (ntypes, ntypes) arrays or callables (dompap/Simulation.py:469-525)."""
        d = self.__dict__
        for name, spec in (("sigma", sigma), ("epsilon", epsilon)):
            if isinstance(spec, (float, int, np.floating, np.integer)) and not isinstance(spec, bool):
                func = _const_func(spec)
            elif isinstance(spec, np.ndarray) or callable(spec):
                if isinstance(spec, np.ndarray):
                    table = spec
                    if table.ndim == 2 and table.shape[0] == table.shape[1]:
                        types = d["_particle_types"]
                        func = (lambda t: (lambda n, m: np.float64(t[types[n, 0], types[m, 0]])))(table)
                    else:
                        raise ValueError(f"Unknown type of {name}: array of shape {table.shape}")
                else:
                    func = spec
            else:
                raise ValueError(f"Unknown type of {name}: {type(spec)}")
            object.__setattr__(self, f"{name}_func", func)
            d[f"_{name}_spec"] = spec
        d["_params_dirty"] = True
        self.set_neighbor_list()

    def scale_box(self, scale_factor: float) -> None:
        """dompap/Simulation.py:527-543."""
        box = self.__getattr__("box_vectors")
        pos = self.__getattr__("positions")
        self.box_vectors = box * scale_factor
        self.positions = pos * scale_factor
        self.set_neighbor_list()

    def get_potential_energy(self) -> float:
        """dompap/Simulation.py:545-592 (all energy methods give the list sum)."""
        if self.energy_method_str not in self._KNOWN_ENERGY_METHODS:
            return None
        self._push()
        e = _lib.ctypes.c_double(0.0)
        _lib.check(self._lib().dp_potential_energy(self._h, _lib.ctypes.byref(e)))
        return float(e.value)

    def get_forces(self) -> np.ndarray:
        """dompap/Simulation.py:594-654 (all force methods give the list sum)."""
        if self.force_method_str not in self._KNOWN_FORCE_METHODS:
            raise ValueError(f"Unknown force method: {self.force_method_str}")
        self._push()
        out = np.empty(self.__dict__["_positions"].shape, dtype=np.float64)
        _lib.check(self._lib().dp_forces(self._h, _lib.dptr(out)))
        return out

    def wrap_into_box(self) -> None:
        """dompap/Simulation.py:656-679 (positions.py:90-98), on the GPU."""
        self._push()
        _lib.check(self._lib().dp_wrap(self._h))
        self._dev_newer.update(("positions", "image_positions"))

    def step(self) -> None:
        """One Langevin G-JF step (dompap/Simulation.py:681-704)."""
        self.run(1)

    def step_leap_frog(self) -> None:
        """One NVE leap-frog step (dompap/Simulation.py:706-724)."""
        self._push()
        self._require_masses()
        _lib.check(self._lib().dp_run(self._h, 1, _lib.DP_INT_NVE))
        self._mark_device_newer()
        self.number_of_steps += 1

    def run(self, steps: int = 1000) -> None:
        """``steps`` G-JF steps on the GPU (dompap/Simulation.py:726-737)."""
        self._push()
        self._require_masses()
        _lib.check(self._lib().dp_run(self._h, int(steps), _lib.DP_INT_GJF))
        self._mark_device_newer()
        self.number_of_steps += int(steps)

    def run_leap_frog(self, steps: int = 1000) -> None:
        """``steps`` NVE leap-frog steps on the GPU (extension)."""
        self._push()
        self._require_masses()
        _lib.check(self._lib().dp_run(self._h, int(steps), _lib.DP_INT_NVE))
        self._mark_device_newer()
        self.number_of_steps += int(steps)

    def set_step_launch(self, lanes_per_particle: int = 0, blocks_per_sm: int = 0) -> None:
        """Launch shape of the fused step kernel (extension; set by
        ``tools.autotune``): lanes per particle 1, 4 or 32 (0: by system size)
        and resident 256-thread CTAs per SM it is compiled for (0: default)."""
        self.__dict__["_step_launch"] = (int(lanes_per_particle), int(blocks_per_sm))
        self._push()
        _lib.check(self._lib().dp_set_step_launch(self._h, int(lanes_per_particle), int(blocks_per_sm)))

    def get_step_launch(self) -> tuple[int, int]:
        """(lanes per particle, resident CTAs per SM) of the fused step in use."""
        self._push()
        lanes, blocks = _lib.ctypes.c_int(0), _lib.ctypes.c_int(0)
        _lib.check(self._lib().dp_get_step_launch(self._h, _lib.ctypes.byref(lanes), _lib.ctypes.byref(blocks)))
        return int(lanes.value), int(blocks.value)

    def run_timed(self, steps: int, kind: str = "gjf") -> float:
        """Run and return the device time in ms (CUDA events on the system's stream)."""
        self._push()
        self._require_masses()
        ms = _lib.ctypes.c_float(0.0)
        k = _lib.DP_INT_GJF if kind == "gjf" else _lib.DP_INT_NVE
        _lib.check(self._lib().dp_run_timed(self._h, int(steps), k, _lib.ctypes.byref(ms)))
        self._mark_device_newer()
        self.number_of_steps += int(steps)
        return float(ms.value)

    def set_integrator(self, time_step: float = None, target_temperature: float = None,
                       temperature_damping_time: float = None) -> None:
        """dompap/Simulation.py:739-759."""
        if time_step is not None:
            self.time_step = np.float64(time_step)
        if target_temperature is not None:
            self.temperature_target = np.float64(target_temperature)
        if temperature_damping_time is not None:
            self.temperature_damping_time = np.float64(temperature_damping_time)
        self.__dict__["_int_dirty"] = True

    def set_precision(self, precision: str) -> None:
        """'fp64' (parity), 'fp32' (float32 pair forces, float64 integration and
        sums) or 'mlp' (the pair surrogate set with set_pair_surrogate)."""
        code = self._KNOWN_PRECISIONS[precision]
        d = self.__dict__
        if code == _lib.DP_PREC_MLP and d.get("_surrogate") is None:
            raise ValueError("set_pair_surrogate() first")
        old = d["_precision"]
        d["_precision"] = code
        if self._h is not None:
            if old == _lib.DP_PREC_MLP or code == _lib.DP_PREC_MLP:
                if old == _lib.DP_PREC_MLP:
                    _lib.check(self._lib().dp_set_precision(self._h, _lib.DP_PREC_FP32))
                d["_pot_dirty"] = True  # the cheap or the full potential source
                if code != _lib.DP_PREC_MLP:
                    _lib.check(self._lib().dp_set_precision(self._h, code))
                self._push()
            else:
                _lib.check(self._lib().dp_set_precision(self._h, code))

    def set_pair_surrogate(self, surrogate) -> None:
        """Evaluate the costly terms of the current pair potential with a trained
        ``dompap_gb300.mlp.PairSurrogate`` (precision 'mlp'); None returns to
        float64 generated code."""
        d = self.__dict__
        if surrogate is None:
            if d["_precision"] == _lib.DP_PREC_MLP:
                self.set_precision("fp64")
            d["_surrogate"] = None
            return
        if surrogate.pair_potential_str != self.pair_potential_str or surrogate.r_cut != float(
                self.pair_potential_r_cut):
            raise ValueError("the surrogate was trained for another pair potential or r_cut")
        if not isinstance(d["_sigma_spec"], (float, int)) or float(d["_sigma_spec"]) != 1.0 or \
                not isinstance(d["_epsilon_spec"], (float, int)) or float(d["_epsilon_spec"]) != 1.0:
            raise ValueError("the pair surrogate needs sigma = epsilon = 1")
        d["_surrogate"] = surrogate
        self.set_precision("mlp")

    def number_of_particles(self) -> int:
        return self.__dict__["_positions"].shape[0]

    def get_number_of_particles(self) -> int:
        return self.__dict__["_positions"].shape[0]

    def get_density(self) -> float:
        return float(self.number_of_particles() / self.get_volume())

    def set_density(self, density: float = 1.0) -> None:
        """dompap/Simulation.py:787-802."""
        dimensions = self.__dict__["_box_vectors"].shape[0]
        current_density = self.get_density()
        scale_factor = (current_density / density) ** (1 / dimensions)
        self.scale_box(scale_factor)

    def get_dimensions_of_space(self) -> int:
        return int(self.__dict__["_box_vectors"].shape[0])

    def _sum_mv2(self) -> float:
        self._push()
        self._require_masses()
        v = _lib.ctypes.c_double(0.0)
        _lib.check(self._lib().dp_sum_mv2(self._h, _lib.ctypes.byref(v)))
        return float(v.value)

    def get_temperature(self) -> float:
        """sum m v^2 / (D N) (dompap/Simulation.py:817-836)."""
        return self._sum_mv2() / (self.get_dimensions_of_space() * self.number_of_particles())

    def get_kinetic_energy(self) -> float:
        """dompap/Simulation.py:896-910."""
        return 0.5 * self._sum_mv2()

    def get_laplacian(self) -> np.ndarray:
        """dompap/Simulation.py:1205-1229."""
        self._push()
        out = np.empty(self.number_of_particles(), dtype=np.float64)
        _lib.check(self._lib().dp_laplacian(self._h, _lib.dptr(out)))
        return out

    def get_configurational_temperature(self) -> float:
        """<|F|^2> / <laplacian> (dompap/Simulation.py:838-856)."""
        forces = self.get_forces()
        numerator = np.mean(np.sum(forces ** 2, axis=1))
        denominator = np.mean(self.get_laplacian())
        return float(numerator / denominator)

    def get_virial(self) -> float:
        """dompap/Simulation.py:946-967 (from the neighbour list; equal to the all-pairs sum)."""
        self._push()
        w = _lib.ctypes.c_double(0.0)
        _lib.check(self._lib().dp_virial(self._h, _lib.ctypes.byref(w)))
        return float(w.value)

    def get_pressure(self) -> float:
        """W/V + sum m v^2 / (D V) (dompap/Simulation.py:969-988)."""
        volume = self.get_volume()
        virial = self.get_virial()
        dims = self.get_dimensions_of_space()
        return float(virial / volume + self._sum_mv2() / dims / volume)

    def get_volume(self) -> float:
        return float(np.prod(self.__dict__["_box_vectors"]))

    def get_diameters(self) -> np.ndarray:
        n = self.number_of_particles()
        diameters = np.ones((n, 1), dtype=np.float64)
        for i in range(n):
            diameters[i] = self.sigma_func(i, i)
        return diameters

    def get_time(self) -> float:
        return float(self.number_of_steps * self.time_step)

    def get_radial_distribution_function(self, r_bins: np.ndarray, type_a: int = -1, type_b: int = -1):
        """g(r) from a GPU pair-distance histogram (dompap/Simulation.py:858-881,
        positions.py:58-87): all ordered pairs including self pairs, np.round
        minimum image, normalised by N_a * N_b and the D-sphere shell volume.
        ``type_a``/``type_b`` (extension) restrict the pairs to two particle types."""
        from scipy.special import gamma

        r_bins = np.ascontiguousarray(r_bins, dtype=np.float64)
        if not np.all(np.diff(r_bins) >= 0):
            raise ValueError("r_bins array must be sorted in ascending order.")
        self._push()
        nb = r_bins.size - 1
        counts = np.zeros(nb, dtype=np.uint64)
        _lib.check(self._lib().dp_rdf_counts(self._h, int(type_a), int(type_b), _lib.dptr(r_bins), nb,
                                             counts.ctypes.data_as(_lib.ctypes.POINTER(_lib.ctypes.c_uint64))))
        types = np.asarray(self.__dict__["_particle_types"]).reshape(-1)
        n_a = int(np.sum(types == type_a)) if type_a >= 0 else self.number_of_particles()
        n_b = int(np.sum(types == type_b)) if type_b >= 0 else self.number_of_particles()
        box = self.__dict__["_box_vectors"]
        dims = self.get_dimensions_of_space()
        dr = np.diff(r_bins)
        r_mid = r_bins[:-1] + dr / 2
        surface = 2 * np.pi ** (dims / 2) / gamma(dims / 2)
        shell = surface * r_mid ** (dims - 1) * dr
        g = counts.astype(np.float64) / shell / (n_a * n_b) * np.prod(box)
        return r_mid, g

    # ------------------------------------------------------------------ I/O
    def to_disk(self, particle_data="simulation.csv", meta_data="simulation.toml") -> None:
        from .io import to_disk

        to_disk(self, particle_data, meta_data)

    def from_disk(self, particle_data="simulation.csv", meta_data="simulation.toml", verbose=False,
                  set_only_particle_data=False) -> dict:
        from .io import from_disk

        return from_disk(self, particle_data, meta_data, verbose, set_only_particle_data)

    def __del__(self):
        h = self.__dict__.get("_h")
        if h is not None:
            try:
                _lib.load().dp_destroy(h)
            except Exception:
                pass
            self.__dict__["_h"] = None
