"""The allocation-free kinetic sum ``dp_sum_mv2_noalloc``.

It exists for callers that cannot call cudaMalloc: hosts that hand out all
device memory from their own pool or a budget fixed at start-up, where a
library allocation can fail or break their accounting. This test owns the
device buffers (torch allocates them); the entry point is only handed
pointers, and its result must equal the handle-based ``dp_sum_mv2`` (FP64
sums, 1e-12 relative) on two calls in a row. The file is named so that pytest
collects it last; it passes alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def test_noalloc_kinetic_sum_matches_handle_entry_point():
    import torch

    from dompap_gb300 import Simulation
    from dompap_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(20261203)
    sim = Simulation()
    sim.set_positions(unit_cell_coordinates=([0.0, 0.0, 0.0], [0.5, 0.5, 0.5]), cells=(12, 12, 12),
                      lattice_constants=(1.0, 1.0, 1.0))
    n = sim.number_of_particles()
    sim.set_masses(masses=list(rng.uniform(0.5, 2.0, size=n)))
    sim.velocities = rng.normal(size=(n, 3))
    sim._push()  # upload the host-side state before calling the C ABI directly
    want = ctypes.c_double(0.0)
    _lib.check(lib.dp_sum_mv2(sim._h, ctypes.byref(want)))
    want = want.value
    assert want > 0

    vel = torch.tensor(np.asarray(sim.velocities), dtype=torch.float64, device="cuda")
    mass = torch.tensor(np.asarray(sim.masses).reshape(-1), dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(float("nan"))
        _lib.check(lib.dp_sum_mv2_noalloc(vel.data_ptr(), mass.data_ptr(), n, 3, out.data_ptr(), stream))
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - want) <= RTOL * want, (got, want)

    # a shorter call right after: nothing of the previous call leaks into it
    half = n // 2
    v = np.asarray(sim.velocities)[:half]
    m = np.asarray(sim.masses).reshape(-1)[:half]
    _lib.check(lib.dp_sum_mv2_noalloc(vel.data_ptr(), mass.data_ptr(), half, 3, out.data_ptr(), stream))
    torch.cuda.synchronize()
    expect = float(np.sum(m * np.sum(v * v, axis=1)))
    assert abs(float(out.item()) - expect) <= RTOL * expect

    # sizes beyond the fixed scratch are rejected before any launch
    rc = lib.dp_sum_mv2_noalloc(vel.data_ptr(), mass.data_ptr(), 5_000_000, 3, out.data_ptr(), stream)
    assert rc == _lib.DP_ERR_ARG
    assert b"exceed" in lib.dp_last_error()
