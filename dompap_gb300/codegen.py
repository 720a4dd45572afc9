"""SymPy pair potential -> CUDA C++ device functions for NVRTC.

Replaces ``make_pair_potential`` (dompap/potential.py:43-66): the expression
string in ``r`` is parsed with SymPy, ``f = -du/dr`` and ``c = d2u/dr2`` are
derived symbolically, and the three are printed as templated device functions

    template <typename R> __device__ R dp_pair_u(R r, R dp_inv_r);   // u(r) - u(r_cut)
    template <typename R> __device__ R dp_pair_f(R r, R dp_inv_r);   // -du/dr
    template <typename R> __device__ R dp_pair_c(R r, R dp_inv_r);   // d2u/dr2

that ``pair_kernels.cuh`` inlines into its neighbour loops (the cut ``r >
r_cut -> 0`` is applied there). ``dp_inv_r`` is ``1/r``, which the kernels get
from one reciprocal square root together with ``r``; negative integer powers
of ``r`` are printed as powers of it, so they cost no division. ``R`` is
``double`` in FP64 mode and ``float`` in FP32 mode, so every literal is printed
as ``R(...)``. Integer powers become multiplication chains, half-integer
powers go through ``sqrt``, everything else calls the CUDA math library.

The value shift ``u(r_cut)`` is evaluated the way the reference evaluates it —
the NumPy-lambdified expression at float64 ``r_cut`` — and embedded as an exact
hexadecimal literal.
"""
from __future__ import annotations

import hashlib

import numpy as np
import sympy as sp
from sympy.printing.c import C99CodePrinter

R_SYM = sp.Symbol("r")
_INV = sp.Symbol("dp_inv_r")

HARDCODED = {
    # dompap/potential.py:10-40: 0.5 (1 - r)^2 and 1 - r for r < 1, curvature 0, r_cut 1
    "Harmonic repulsive": ("0.5*(1-r)**2", 1.0),
}

_HARDCODED_SOURCE = """
template <typename R> __device__ __forceinline__ R dp_pair_u(R r, R) { return r < R(1) ? R(0.5) * (R(1) - r) * (R(1) - r) : R(0); }
template <typename R> __device__ __forceinline__ R dp_pair_f(R r, R) { return r < R(1) ? R(1) - r : R(0); }
template <typename R> __device__ __forceinline__ R dp_pair_c(R r, R) { return R(0); }
"""

_PRELUDE = """
template <int N, typename R> __device__ __forceinline__ R dp_ipow(R x) {
    if constexpr (N == 0) { return R(1); }
    else if constexpr (N == 1) { return x; }
    else if constexpr (N % 2 == 0) { const R h = dp_ipow<N / 2, R>(x); return h * h; }
    else { const R h = dp_ipow<N / 2, R>(x); return h * h * x; }
}
"""


def _hex(value: float) -> str:
    value = float(value)
    if np.isnan(value):
        return "R(0.0/0.0)"
    if np.isinf(value):
        return "R(1.0/0.0)" if value > 0 else "R(-1.0/0.0)"
    return f"R({float.hex(value)})"


def _float32_exact(value: float) -> bool:
    """A finite value that float32 holds exactly (normal range or zero)."""
    if not np.isfinite(value):
        return False
    if value == 0.0:
        return True
    return 2.0 ** -126 <= abs(value) < 2.0 ** 127 and float(np.float32(value)) == value


class _CudaPrinter(C99CodePrinter):
    """C99 printer with ``R(...)`` literals and multiplication-chain powers;
    constants float32 holds exactly are printed as ``dp_k<R>(...f)`` (the
    double-float arithmetic multiplies and adds them as single floats)."""

    def _print_Float(self, expr):
        value = float(expr)
        if _float32_exact(value):
            return f"dp_k<R>({float.hex(value)}f)"
        return _hex(value)

    def _print_Integer(self, expr):
        n = int(expr)
        if abs(n) <= 2 ** 24:
            return f"dp_k<R>({float(n)!r}f)"
        return f"R({n})"

    def _print_Rational(self, expr):
        return f"(R({int(expr.p)})/R({int(expr.q)}))"

    def _print_NaN(self, expr):
        return "R(0.0/0.0)"

    def _print_Infinity(self, expr):
        return "R(1.0/0.0)"

    def _print_NegativeInfinity(self, expr):
        return "R(-1.0/0.0)"

    def _print_Pi(self, expr):
        return _hex(np.pi)

    def _print_Exp1(self, expr):
        return _hex(np.e)

    def _print_Pow(self, expr):
        base, exp = expr.base, expr.exp
        b = self._print(base)
        if exp.is_Integer:
            n = int(exp)
            if n == 0:
                return "R(1)"
            if 0 < n <= 64:
                return f"dp_ipow<{n}, R>({b})"
            if -64 <= n < 0:
                return f"(R(1)/dp_ipow<{-n}, R>({b}))"
        if exp.is_Rational and exp.q == 2:
            p = int(exp.p)
            if 0 < p <= 64:
                return f"dp_ipow<{p}, R>(sqrt({b}))"
            if -64 <= p < 0:
                return f"(R(1)/dp_ipow<{-p}, R>(sqrt({b})))"
        if exp == sp.Rational(1, 3):
            return f"cbrt({b})"
        return f"pow({b}, {self._print(exp)})"

    def _print_Abs(self, expr):
        return f"fabs({self._print(expr.args[0])})"


def _share_reciprocal(expr: sp.Expr) -> tuple[sp.Expr, bool]:
    """Rewrite r**(-n) as dp_inv_r**n (1/r is an argument of the device function)."""
    used = False

    def repl(e):
        nonlocal used
        if e.is_Pow and e.base == R_SYM and e.exp.is_Integer and int(e.exp) < 0:
            used = True
            return _INV ** (-int(e.exp))
        return e

    out = expr.replace(lambda e: e.is_Pow and e.base == R_SYM and e.exp.is_Integer and int(e.exp) < 0, repl)
    return out, used


def _horner(expr: sp.Expr) -> sp.Expr:
    """A polynomial in one variable (r or 1/r) in Horner form: the force of
    4 (r^-12 - r^-6), 48 r^-13 - 24 r^-7, becomes r^-7 (48 r^-6 - 24), with
    fewer multiplications; anything else is returned as it is."""
    syms = expr.free_symbols
    if len(syms) != 1:
        return expr
    (x,) = syms
    if not expr.is_polynomial(x):
        return expr
    return sp.horner(sp.expand(expr), wrt=x)


def _function_source(name: str, expr: sp.Expr, shift_literal: str | None = None, horner: bool = False) -> str:
    printer = _CudaPrinter()
    expr, _ = _share_reciprocal(expr)
    if horner:
        expr = _horner(expr)
    repl, reduced = sp.cse(expr, symbols=sp.numbered_symbols("dp_t"))
    lines = [f"template <typename R> __device__ __forceinline__ R {name}(R r, R dp_inv_r) {{"]
    for sym, sub in repl:
        lines.append(f"    const R {sym} = {printer.doprint(sub)};")
    body = printer.doprint(reduced[0])
    if shift_literal is not None:
        body = f"({body}) - {shift_literal}"
    lines.append(f"    return {body};")
    lines.append("}")
    return "\n".join(lines)


def derive(pair_potential_str: str):
    """SymPy u, f = -du/dr, c = d2u/dr2 (dompap/potential.py:47-51)."""
    u = sp.sympify(pair_potential_str)
    f = sp.diff(-u, R_SYM)
    c = sp.diff(u, R_SYM, 2)
    return u, f, c


def value_at_cut(pair_potential_str: str, r_cut: float) -> float:
    """u(r_cut) as the reference computes its shift (lambdified NumPy, float64)."""
    u = sp.sympify(pair_potential_str)
    fn = sp.lambdify(R_SYM, u, "numpy")
    with np.errstate(all="ignore"):
        return float(np.float64(fn(np.float64(r_cut))))


def make_pair_source(pair_potential_str: str, r_cut: float) -> tuple[str, float]:
    """CUDA source of dp_pair_u/f/c for a SymPy expression in ``r``; returns
    ``(source, r_cut)``. Hard-coded names (``'Harmonic repulsive'``) map to
    their fixed form and cutoff, as dompap/Simulation.py:434-441 does."""
    if pair_potential_str in HARDCODED:
        return _PRELUDE + _HARDCODED_SOURCE, HARDCODED[pair_potential_str][1]
    u, f, c = derive(pair_potential_str)
    free = (u.free_symbols | f.free_symbols | c.free_symbols) - {R_SYM}
    if free:
        raise ValueError(f"pair potential has symbols other than r: {sorted(map(str, free))}")
    shift = value_at_cut(pair_potential_str, r_cut)
    src = "\n".join([
        _PRELUDE,
        f"// u(r) = {pair_potential_str}   (r_cut = {r_cut!r}, u(r_cut) = {shift!r})",
        _function_source("dp_pair_u", u, shift_literal=_hex(shift)),
        _function_source("dp_pair_f", f, horner=True),
        _function_source("dp_pair_c", c),
    ])
    return src, float(r_cut)


def source_hash(src: str) -> str:
    return hashlib.sha1(src.encode()).hexdigest()[:12]
