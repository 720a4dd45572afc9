"""The benchmark's host-side pieces (no GPU): the costly test potential of
the surrogate workload is force-shifted to zero at r_cut, and its added
costly terms are classified as costly by the surrogate's term split."""
import os
import sys

import sympy as sp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, REPO)
    import bench

    return bench


def test_costly_potential_is_force_shifted_at_r_cut():
    bench = _bench()
    r = sp.symbols("r")
    for m in (0, 4):
        u = sp.sympify(bench.expensive_string(3.0, m))
        assert abs(float(u.subs(r, 3.0))) < 1e-12
        assert abs(float(sp.diff(u, r).subs(r, 3.0))) < 1e-12


def test_added_terms_are_costly():
    from dompap_gb300.mlp import split_costly

    bench = _bench()
    r = sp.symbols("r")
    base_cheap, base_costly = split_costly(bench.expensive_string(3.0, 0))
    cheap, costly = split_costly(bench.expensive_string(3.0, 8))
    # the cheap part changes only by the shift's constant and linear term
    assert sp.Poly(sp.expand(sp.sympify(cheap) - sp.sympify(base_cheap)), r).degree() <= 1
    extra = sp.Add.make_args(sp.expand(sp.sympify(costly) - sp.sympify(base_costly), deep=False))
    assert len(extra) == 8 and all(t.has(sp.exp) and t.has(sp.cos) for t in extra)
    assert abs(float((sp.sympify(costly) - sp.sympify(base_costly)).subs(r, 1.3))) > 0
