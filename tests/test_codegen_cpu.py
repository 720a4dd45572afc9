"""The SymPy -> CUDA printer (dompap/potential.py:43-66 restated as device
code): derivatives, constants, Horner forms and the value shift, checked on
the host by evaluating the printed expressions with Python semantics."""
import math
import re

import pytest
import sympy as sp

from dompap_gb300 import codegen


def _body(src, name):
    m = re.search(r"R %s\(R r, R dp_inv_r\) \{\n(.*?)\n\}" % name, src, re.S)
    assert m, name
    return m.group(1)


def _evaluate(body, r):
    """Run a printed function body for R = float (Python) at r."""
    py = body.replace("template <typename R>", "")
    env = {"r": r, "dp_inv_r": 1.0 / r, "exp": math.exp, "cos": math.cos, "sin": math.sin, "sqrt": math.sqrt,
           "pow": math.pow, "log": math.log}
    lines = []
    for line in py.strip().splitlines():
        line = line.strip().rstrip(";")
        line = re.sub(r"dp_k<R>\(([^)]*?)f\)", lambda m: repr(float.fromhex(m.group(1)) if m.group(1).startswith(("0x", "-0x")) else float(m.group(1))), line)
        line = re.sub(r"R\((-?0x[0-9a-fp.+-]+)\)", lambda m: repr(float.fromhex(m.group(1))), line)
        line = re.sub(r"R\((-?\d+)\)", r"\1.0", line)
        line = re.sub(r"dp_ipow<(\d+), R>\(", r"_ipow(\1, ", line)
        if line.startswith("const R "):
            name, expr = line[len("const R "):].split(" = ", 1)
            lines.append(f"{name} = {expr}")
        elif line.startswith("return "):
            lines.append(f"_out = {line[len('return '):]}")
    env["_ipow"] = lambda n, x: x ** n
    exec("\n".join(lines), env)
    return env["_out"]


@pytest.mark.parametrize("pot, rc", [("4*(r**-12-r**-6)", 2.5), ("(1-r)**2", 1.0),
                                     ("4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r)", 3.0)])
def test_printed_functions_match_sympy(pot, rc):
    src, r_cut = codegen.make_pair_source(pot, rc)
    assert r_cut == rc
    r = sp.Symbol("r")
    u = sp.sympify(pot)
    f = sp.diff(-u, r)
    c = sp.diff(u, r, 2)
    shift = codegen.value_at_cut(pot, rc)
    for x in (0.9, 1.1, 1.7, 2.4):
        if x > rc:
            continue
        want_u = float(u.subs(r, x)) - shift
        want_f = float(f.subs(r, x))
        want_c = float(c.subs(r, x))
        assert _evaluate(_body(src, "dp_pair_u"), x) == pytest.approx(want_u, rel=1e-12, abs=1e-12)
        assert _evaluate(_body(src, "dp_pair_f"), x) == pytest.approx(want_f, rel=1e-12, abs=1e-12)
        assert _evaluate(_body(src, "dp_pair_c"), x) == pytest.approx(want_c, rel=1e-12, abs=1e-12)


def test_constants_and_horner_form():
    src, _ = codegen.make_pair_source("4*(r**-12-r**-6)", 2.5)
    f = _body(src, "dp_pair_f")
    # the LJ force 48 r^-13 - 24 r^-7 in Horner form, constants float32-exact
    assert "dp_ipow<7, R>(dp_inv_r)*(dp_k<R>(48.0f)*dp_ipow<6, R>(dp_inv_r) + dp_k<R>(-24.0f))" in f
    # a constant float32 cannot hold stays a float64 literal
    src2, _ = codegen.make_pair_source("0.1*r**2", 1.0)
    assert "R(0x1.999999999999ap-4)" in src2 or "R(0x1.999999999999ap-3)" in src2
    # non-polynomial expressions are printed as derived
    src3, _ = codegen.make_pair_source("exp(-r)", 2.0)
    assert "exp(" in _body(src3, "dp_pair_f")


def test_rejects_foreign_symbols():
    with pytest.raises(ValueError):
        codegen.make_pair_source("r**2 + a", 1.0)


def test_surrogate_split_of_a_potential():
    """The surrogate learns only the costly terms (exp, cos, non-integer
    powers); the cheap ones stay generated code, and the two add up to the
    potential."""
    from dompap_gb300.mlp import split_costly

    pot = "4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r) - 0.25 - (r - 3.0)*0.125"
    cheap, costly = split_costly(pot)
    r = sp.Symbol("r")
    assert sp.simplify(sp.sympify(cheap) + sp.sympify(costly) - sp.sympify(pot)) == 0
    assert not sp.sympify(cheap).has(sp.exp, sp.cos)
    assert sp.sympify(costly).has(sp.exp) and sp.sympify(costly).has(sp.cos)
    assert sp.sympify(costly).free_symbols == {r}
    cheap2, costly2 = split_costly("r**0.5 + r**-6")
    assert sp.sympify(costly2) == sp.sympify("r**0.5") and sp.sympify(cheap2) == sp.sympify("r**-6")
