"""Oracle for the dompap molecular-dynamics hot path — TEST INFRASTRUCTURE ONLY.

This package is the checker, never the product. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` may import it. The product path (``dompap_gb300``) never imports,
links or executes anything from here, and it fails loudly when its CUDA library
is missing.

Contents
--------
``numpy_ref``
    A NumPy restatement of the reference's float64 arithmetic for the path
    (pair potential from SymPy, single-shift minimum image, double-loop
    neighbour list, neighbour-list force / energy / Laplacian, double-loop
    virial, G-JF Langevin and NVE leap-frog steps, wrap into box, skin
    trigger, radial distribution function). Every function cites the
    reference ``file:line`` it follows. Pair sets and per-pair values are
    bit-identical to the reference; sums are taken in the reference's
    sequential order.
``cport``
    A C/OpenMP restatement of the same loops (the "Numba-equivalent" CPU
    baseline timed beside the GPU), built by ``oracle/cport/build.py``.
``stubs``
    ``numba`` / ``toml`` / ``matplotlib`` stand-ins that let the UNMODIFIED
    reference package be imported where Numba is absent (used only by
    ``tests/golden/make_golden.py`` to produce the committed fixtures).

Parity is pinned: ``tests/test_oracle_golden.py`` checks ``numpy_ref`` against
golden vectors produced by running the unmodified reference
(``tests/golden/make_golden.py``) and against the reference's own test values.
"""
