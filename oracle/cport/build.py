"""Build the C/OpenMP restatement (``md_port.c``) and per-potential pair
functions — benchmark/test infrastructure only (never used by the product).

``build()`` compiles ``oracle/_ref``-free ``oracle/cport/_build/libmdport.so``
with gcc. ``compile_potential(expr, r_cut)`` prints the SymPy force
``f = -du/dr`` as C (``sympy.ccode``), wraps it with the reference's cut
``r > r_cut -> 0`` (dompap/potential.py:64) and compiles it into its own small
shared library, returning the function pointer for ``dp_port_forces`` — the
analogue of the reference handing its jitted closure to its force loop.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmdport.so")
CFLAGS = ["-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "md_port.c")
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", *CFLAGS, src, "-o", tmp, "-lm"], check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


_PAIR_FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double)
_loaded = {}


def load():
    if "lib" in _loaded:
        return _loaded["lib"]
    if not os.path.exists(LIB):
        build()
    lib = ctypes.CDLL(LIB)
    d, i32, i64 = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32), ctypes.c_int64
    lib.dp_port_threads.restype = ctypes.c_int
    lib.dp_port_nl_double_loop.restype = i64
    lib.dp_port_nl_double_loop.argtypes = [d, i64, ctypes.c_int, d, ctypes.c_double, ctypes.c_int, i32]
    lib.dp_port_nl_cell_list_3d.restype = i64
    lib.dp_port_nl_cell_list_3d.argtypes = [d, i64, d, ctypes.c_double, ctypes.c_int, i32]
    lib.dp_port_nl_is_old.restype = ctypes.c_int
    lib.dp_port_nl_is_old.argtypes = [d, d, i64, ctypes.c_int, d, ctypes.c_double]
    lib.dp_port_forces.restype = None
    lib.dp_port_forces.argtypes = [d, i64, ctypes.c_int, d, i32, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                   ctypes.c_double, d]
    lib.dp_port_forces_types.restype = None
    lib.dp_port_forces_types.argtypes = [d, i64, ctypes.c_int, d, i32, ctypes.c_int, ctypes.c_void_p, i32,
                                         ctypes.c_int, d, d, d]
    lib.dp_port_gjf.restype = None
    lib.dp_port_gjf.argtypes = [d, d, d, d, d, i64, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, d]
    lib.dp_port_wrap.restype = None
    lib.dp_port_wrap.argtypes = [d, i32, i64, ctypes.c_int, d]
    lib.dp_port_seed.argtypes = [ctypes.c_uint64]
    _loaded["lib"] = lib
    return lib


def compile_potential(pair_potential_str: str, r_cut: float) -> int:
    """Address of ``double f(double r)`` for the SymPy potential (cut at r_cut)."""
    import sympy as sp

    r = sp.Symbol("r")
    f = sp.diff(-sp.sympify(pair_potential_str), r)
    body = sp.ccode(f, standard="C99")
    rc = "INFINITY" if r_cut == float("inf") else repr(float(r_cut))
    code = f"#include <math.h>\ndouble dp_port_pair_force(double r) {{ return r > {rc} ? 0.0 : ({body}); }}\n"
    key = hashlib.sha1(code.encode()).hexdigest()[:16]
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, f"pot_{key}.so")
    if not os.path.exists(so):
        c = os.path.join(BUILD, f"pot_{key}.c")
        with open(c, "w") as fh:
            fh.write(code)
        subprocess.run(["gcc", *CFLAGS, c, "-o", so + ".tmp", "-lm"], check=True, capture_output=True, text=True)
        os.replace(so + ".tmp", so)
    if so not in _loaded:
        _loaded[so] = ctypes.CDLL(so)
    return ctypes.cast(_loaded[so].dp_port_pair_force, ctypes.c_void_p).value
