"""The C/OpenMP restatement (``oracle/cport``) — the CPU baseline and the
reference arm of bench.py — against the reference's own outputs
(``tests/golden``) and the NumPy oracle: pair sets bit-exact, forces to
rounding, the skin trigger, the wrap and the G-JF update. CPU only."""
import ctypes

import numpy as np
import pytest

from conftest import config_of
from oracle import numpy_ref as ref

cport = pytest.importorskip("oracle.cport.build")


def _ptr(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


@pytest.fixture(scope="module")
def lib():
    return cport.load()


def test_double_loop_list_and_forces_match_the_reference(lib, golden_configs):
    c = config_of(golden_configs, "lj500")
    pos = np.ascontiguousarray(c["positions"], dtype=np.float64)
    box = np.ascontiguousarray(c["box"], dtype=np.float64)
    n, dim = pos.shape
    kmax = int(c["kmax"])
    cutoff = float(c["r_cut"]) + float(c["skin"])
    nl = np.empty((n, kmax), dtype=np.int32)
    lib.dp_port_nl_double_loop(_ptr(pos), n, dim, _ptr(box), cutoff, kmax, _ptr(nl, ctypes.c_int32))
    want_nl = c["nlist"]  # stored up to its longest row
    k = want_nl.shape[1]
    assert np.array_equal(nl[:, :k], want_nl) and np.all(nl[:, k:] == -1)
    fptr = cport.compile_potential(str(c["pot"]), float(c["r_cut"]))
    out = np.empty_like(pos)
    lib.dp_port_forces(_ptr(pos), n, dim, _ptr(box), _ptr(nl, ctypes.c_int32), kmax, fptr, 1.0, 1.0, _ptr(out))
    want = c["forces"]
    assert np.sqrt(np.mean((out - want) ** 2) / np.mean(want ** 2)) <= 1e-13


def test_skin_trigger_matches_the_reference(lib, golden_unit):
    pos = np.array([[0, 0, 0], [1, 1, 1]], dtype=np.float64)
    old = np.array([[0.5, 0, 0], [1, 1, 1]], dtype=np.float64)
    box = np.array([5.0] * 3)
    got = [bool(lib.dp_port_nl_is_old(_ptr(pos), _ptr(old), 2, 3, _ptr(box), float(s))) for s in golden_unit["skin/skins"]]
    assert got == [bool(x) for x in golden_unit["skin/is_old"]]


def test_wrap_matches_the_reference(lib, golden_unit):
    pos = np.ascontiguousarray(golden_unit["wrap/in"], dtype=np.float64).copy()
    n, dim = pos.shape
    img = np.zeros((n, dim), dtype=np.int32)
    box = np.array([2.0] * dim)  # the box the fixture was written with (tests/test_positions.py:78-93)
    lib.dp_port_wrap(_ptr(pos), _ptr(img, ctypes.c_int32), n, dim, _ptr(box))
    assert np.array_equal(pos, golden_unit["wrap/positions"])
    assert np.array_equal(img, golden_unit["wrap/images"])


def test_gjf_without_noise_matches_the_oracle(lib, golden_unit):
    pos = np.ascontiguousarray(golden_unit["gjf/positions"], dtype=np.float64).copy()
    vel = np.ascontiguousarray(golden_unit["gjf/velocities"], dtype=np.float64).copy()
    beta = np.ascontiguousarray(golden_unit["gjf/betas"], dtype=np.float64).copy()
    force = np.ascontiguousarray(golden_unit["gjf/forces"], dtype=np.float64)
    mass = np.ascontiguousarray(golden_unit["gjf/masses"], dtype=np.float64).reshape(-1)
    n, dim = pos.shape
    # tau = inf: alpha = 0, no new noise; the old betas still enter b (beta_old + 0) / (2m)
    want = ref.gjf_step(pos.copy(), vel.copy(), beta.copy(), force, mass.reshape(n, 1), 0.005, 1.3, np.inf,
                        np.zeros_like(pos))
    scratch = np.empty(n * dim)
    lib.dp_port_gjf(_ptr(pos), _ptr(vel), _ptr(beta), _ptr(force), _ptr(mass), n, dim, 0.005, 1.3, np.inf,
                    _ptr(scratch))
    assert np.max(np.abs(pos - want[0])) <= 1e-14
    assert np.max(np.abs(vel - want[1])) <= 1e-14


def test_type_table_forces_match_the_reference(lib, golden_configs):
    """The binary mixture with sigma/epsilon per type pair (the reference's
    index callables over a type table): forces to rounding."""
    c = config_of(golden_configs, "wahn")
    pos = np.ascontiguousarray(c["positions"], dtype=np.float64)
    box = np.ascontiguousarray(c["box"], dtype=np.float64)
    n, dim = pos.shape
    kmax = int(c["kmax"])
    types = np.ascontiguousarray(c["types"].reshape(-1), dtype=np.int32)
    sig = np.ascontiguousarray(c["sigma_table"], dtype=np.float64)
    eps = np.ascontiguousarray(c["epsilon_table"], dtype=np.float64)
    cutoff = float(np.max(sig)) * float(c["r_cut"]) + float(c["skin"])
    nl = np.empty((n, kmax), dtype=np.int32)
    lib.dp_port_nl_double_loop(_ptr(pos), n, dim, _ptr(box), cutoff, kmax, _ptr(nl, ctypes.c_int32))
    k = c["nlist"].shape[1]
    assert np.array_equal(nl[:, :k], c["nlist"]) and np.all(nl[:, k:] == -1)
    fptr = cport.compile_potential(str(c["pot"]), float(c["r_cut"]))
    out = np.empty_like(pos)
    lib.dp_port_forces_types(_ptr(pos), n, dim, _ptr(box), _ptr(nl, ctypes.c_int32), kmax, fptr,
                             _ptr(types, ctypes.c_int32), sig.shape[0], _ptr(sig), _ptr(eps), _ptr(out))
    want = c["forces"]
    assert np.sqrt(np.mean((out - want) ** 2) / np.mean(want ** 2)) <= 1e-13
