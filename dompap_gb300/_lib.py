"""ctypes binding of ``libdompap_gpu.so`` (the C ABI in ``include/dompap_gpu.h``).

The library is built in-tree by ``dompap_gb300._build`` (``__graft_entry__.build()``).
There is no CPU fallback: if the library is missing or cannot be loaded, every
entry point raises ``DompapGPUError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdompap_gpu.so")

DP_OK = 0
DP_ERR_ARG = 1
DP_ERR_CUDA = 2
DP_ERR_NVRTC = 3
DP_ERR_OVERFLOW = 4
DP_ERR_GEOMETRY = 5
DP_ERR_NONFINITE = 6
DP_ERR_NOPOT = 7
DP_ERR_TIMEOUT = 8

DP_METHOD_LIST = 0
DP_METHOD_ALLPAIRS = 1
DP_METHOD_ALLPAIRS_NEWTON = 2
DP_PREC_FP64 = 0
DP_PREC_FP32 = 1
DP_PREC_MLP = 2
DP_NL_CELL = 0
DP_NL_ALLPAIRS = 1
DP_INT_GJF = 0
DP_INT_NVE = 1
DP_PAIR_CONST = 0
DP_PAIR_TYPES = 1
DP_PAIR_DENSE = 2
DP_KERNEL_FORCES = 0
DP_KERNEL_GJF = 1
DP_KERNEL_NVE = 2
DP_KERNEL_REBUILD = 3
DP_KERNEL_SKIN = 4
DP_KERNEL_STEP = 5

_ERROR_NAMES = {
    DP_ERR_ARG: "invalid argument",
    DP_ERR_CUDA: "CUDA error",
    DP_ERR_NVRTC: "pair-potential compilation failed",
    DP_ERR_OVERFLOW: "neighbour-list overflow",
    DP_ERR_GEOMETRY: "invalid geometry",
    DP_ERR_NONFINITE: "non-finite force or position",
    DP_ERR_NOPOT: "no pair potential",
    DP_ERR_TIMEOUT: "device-side wait timed out",
}


class DompapGPUError(RuntimeError):
    """A failure reported by the CUDA library (its status code is ``.code``)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERROR_NAMES.get(code, 'error')} ({code}): {message}")
        self.code = code


class DpStats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int64),
        ("rebuilds", ctypes.c_int64),
        ("max_neighbors", ctypes.c_int32),
        ("neighbor_capacity", ctypes.c_int32),
        ("cells", ctypes.c_int32 * 4),
        ("cell_capacity", ctypes.c_int32),
        ("method_used", ctypes.c_int32),
        ("nl_cutoff", ctypes.c_double),
        ("conditional_graphs", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes)
_SIGNATURES = {
    "dp_last_error": (ctypes.c_char_p, []),
    "dp_version": (ctypes.c_int, []),
    "dp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(_P)]),
    "dp_destroy": (ctypes.c_int, [_P]),
    "dp_set_precision": (ctypes.c_int, [_P, ctypes.c_int]),
    "dp_set_positions": (ctypes.c_int, [_P, _D]),
    "dp_get_positions": (ctypes.c_int, [_P, _D]),
    "dp_set_velocities": (ctypes.c_int, [_P, _D]),
    "dp_get_velocities": (ctypes.c_int, [_P, _D]),
    "dp_set_betas": (ctypes.c_int, [_P, _D]),
    "dp_get_betas": (ctypes.c_int, [_P, _D]),
    "dp_set_images": (ctypes.c_int, [_P, _I32]),
    "dp_get_images": (ctypes.c_int, [_P, _I32]),
    "dp_set_masses": (ctypes.c_int, [_P, _D]),
    "dp_set_types": (ctypes.c_int, [_P, _I32]),
    "dp_set_box": (ctypes.c_int, [_P, _D]),
    "dp_set_potential": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_double]),
    "dp_set_pair_params": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _D, _D]),
    "dp_set_neighbor_list": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    "dp_update_neighbor_list": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "dp_get_neighbor_list": (ctypes.c_int, [_P, _I32, ctypes.c_int, ctypes.POINTER(ctypes.c_int32)]),
    "dp_get_reference_positions": (ctypes.c_int, [_P, _D]),
    "dp_set_integrator": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]),
    "dp_run": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int]),
    "dp_selftest_bounded_wait": (ctypes.c_int, [_P, ctypes.c_int32]),
    "dp_run_host": (ctypes.c_int, [_P, _D, _D, _D, ctypes.c_int64, ctypes.c_int, _D, _D, _D]),
    "dp_run_timed": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "dp_forces": (ctypes.c_int, [_P, _D]),
    "dp_potential_energy": (ctypes.c_int, [_P, _D]),
    "dp_virial": (ctypes.c_int, [_P, _D]),
    "dp_laplacian": (ctypes.c_int, [_P, _D]),
    "dp_sum_mv2": (ctypes.c_int, [_P, _D]),
    "dp_eval_potential": (ctypes.c_int, [_P, _D, ctypes.c_int64, _D, _D, _D]),
    "dp_get_normals": (ctypes.c_int, [_P, ctypes.c_int64, _D]),
    "dp_wrap": (ctypes.c_int, [_P]),
    "dp_rdf_counts": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint64)]),
    "dp_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(DpStats)]),
    "dp_time_kernel": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "dp_kernel_launches": (ctypes.c_int64, [_P]),
    "dp_set_step_launch": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "dp_set_pair_methods": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "dp_get_step_launch": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "dp_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _I32, ctypes.POINTER(_P)]),
    "dp_batch_destroy": (ctypes.c_int, [_P]),
    "dp_batch_set_state": (ctypes.c_int, [_P, _D, _D, _D, _D]),
    "dp_batch_get_state": (ctypes.c_int, [_P, _D, _D, _I32]),
    "dp_batch_set_potential": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_double]),
    "dp_batch_set_integrator": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_uint64]),
    "dp_batch_set_launch": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "dp_batch_run": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_float)]),
    "dp_batch_set_neighbor_list": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_int]),
    "dp_nvrtc_check": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                      ctypes.POINTER(ctypes.c_int64)]),
    "dp_nvrtc_resources": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                          ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "dp_batch_list_stats": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_int32)]),
    "dp_batch_observables": (ctypes.c_int, [_P, _D, ctypes.c_int]),
    "dp_batch_last_forces": (ctypes.c_int, [_P, _D]),
    "dp_mlp_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "dp_mlp_destroy": (ctypes.c_int, [_P]),
    "dp_mlp_param_count": (ctypes.c_int, []),
    "dp_mlp_set_params": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "dp_mlp_get_params": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    "dp_mlp_set_data": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                       ctypes.c_int64]),
    "dp_mlp_train": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "dp_mlp_eval": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), ctypes.c_int64,
                                   ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "dp_mlp_gradients": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                        ctypes.c_int64, ctypes.c_float, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_float)]),
    "dp_set_mlp": (ctypes.c_int, [_P, _P]),
    "dp_sum_mv2_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]),
}

_lib = None
_lib_lock = threading.Lock()


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library (once); raises if it is missing or does not load."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise DompapGPUError(DP_ERR_CUDA, f"{path} is missing: build it with "
                                 "`python -c 'import __graft_entry__ as g; g.build()'` "
                                 "(or `python -m dompap_gb300._build`)")
        try:
            lib = ctypes.CDLL(path)
        except OSError as exc:
            raise DompapGPUError(DP_ERR_CUDA, f"cannot load {path}: {exc}") from exc
        for name, (restype, argtypes) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(rc: int) -> None:
    if rc != DP_OK:
        msg = load().dp_last_error().decode(errors="replace")
        raise DompapGPUError(rc, msg)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_D)


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_I32)
