"""A short test run of the default system (dompap/tools/run_test_simulation.py:7-28)."""
from __future__ import annotations

from time import perf_counter

from .autotune import autotune
from .progress_bar import progress_bar


def run_test_simulation(verbose: bool = False):
    """The default ``Simulation``, autotuned, then 1000 steps (the progress bar
    every 10 steps when ``verbose``); returns the simulation."""
    from ..simulation import Simulation

    if verbose:
        print("  ..:: Run test simulation ::..")
    tic = perf_counter()
    sim = Simulation()
    toc = perf_counter()
    if verbose:
        print(f"Simulation initialization took {toc - tic:.3f} seconds")
    sim = autotune(sim, verbose=verbose)
    steps, stride = 1000, 10
    for step in range(steps):
        sim.step()
        if step % stride == 0 and verbose:
            progress_bar(step, steps, stride)
    if verbose:
        progress_bar(steps, steps, stride, finalize=True)
    return sim
