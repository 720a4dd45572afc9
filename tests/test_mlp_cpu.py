"""Host-side logic of the pair surrogate (no GPU): the split of a potential
into cheap and costly terms and the tanh grid that starts layer 1."""
import numpy as np

from dompap_gb300 import mlp


def test_split_costly_terms():
    import sympy as sp

    r = sp.symbols("r")
    cheap, costly = mlp.split_costly("4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r)")
    assert sp.simplify(sp.sympify(cheap) - (4 * r ** -12 - 4 * r ** -6)) == 0
    want = sp.Rational(1, 2) * sp.exp(-50 * (r - sp.Rational(3, 2)) ** 2) + sp.Rational(1, 10) * sp.cos(4 * r) * sp.exp(-r)
    assert abs(float((sp.sympify(costly) - want).subs(r, 1.37))) < 1e-12


def test_tanh_grid_places_units_where_the_target_bends():
    x = np.linspace(-1.0, 2.0, 4001)
    x0 = 0.3
    y = (x - x0) * np.exp(-((x - x0) ** 2) / 0.005)  # a narrow feature at x0
    w, b = mlp.tanh_grid(x, y, np.random.default_rng(0))
    c = -b / w
    assert w.shape == b.shape == (64,)
    assert np.all(np.diff(c) > 0) and c[0] >= x[0] and c[-1] <= x[-1]
    # slope 0.7 / local spacing of the centres, either sign
    assert np.allclose(np.abs(w) * np.gradient(c), 0.7)
    assert {1.0, -1.0} == set(np.sign(w))
    # far more units near the feature than an even spread (64 x 0.4 / 3 ~ 8.5)
    assert np.sum(np.abs(c - x0) < 0.2) >= 20


def test_tanh_grid_is_even_for_constant_curvature():
    x = np.linspace(0.0, 4.0, 4001)
    w, b = mlp.tanh_grid(x, 3.0 * x * x + 1.0, np.random.default_rng(1))
    c = -b / w
    assert np.allclose(np.diff(c), 4.0 / 64, rtol=1e-2)
