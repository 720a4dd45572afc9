"""Host-side logic of the batched replicas (no GPU): the near-cubic fcc cell
counts and the seeded replica specs of the 4,096-system LJ workload."""
import itertools

import numpy as np

from dompap_gb300.batched import fcc_cells_for, lj_replica_specs


def test_fcc_cells_are_near_cubic_and_closest():
    for n in (64, 100, 500, 864, 1000, 2048, 4000, 8192):
        cells = fcc_cells_for(n)
        assert max(cells) - min(cells) <= 1 and list(cells) == sorted(cells, reverse=True)
        # no near-cubic box (sides k-1..k+1, differing by at most one) is closer to n
        k = max(1, int(round((n / 4.0) ** (1.0 / 3.0))))
        best = min(abs(4 * a * b * c - n) for a, b, c in itertools.product((k - 1, k, k + 1), repeat=3)
                   if min(a, b, c) >= 1 and max(a, b, c) - min(a, b, c) <= 1)
        assert abs(4 * int(np.prod(cells)) - n) == best


def test_lj_replica_specs_follow_the_workload():
    r_cut, density = 2.5, 0.8442
    specs, rejected = lj_replica_specs(n_rep=200, seed=3)
    again, rejected2 = lj_replica_specs(n_rep=200, seed=3)
    assert len(specs) == 200 and rejected == rejected2 >= 0
    counts = np.array([s.positions.shape[0] for s in specs])
    assert np.all(counts % 4 == 0) and counts.min() >= 4 and counts.max() <= 4 * 14 ** 3
    for s, t in zip(specs, again):
        assert np.array_equal(s.positions, t.positions) and np.array_equal(s.velocities, t.velocities)
        n = s.positions.shape[0]
        assert s.positions.shape == s.velocities.shape == (n, 3)
        assert np.min(s.box) >= 2 * r_cut
        assert abs(n / np.prod(s.box) - density) <= 1e-12 * density
        assert np.all(s.positions >= 0.0) and np.all(s.positions < s.box)
        assert 0.7 <= s.temperature <= 2.0
    # N log-uniform over [64, 8192]: the median near the geometric mean 724
    assert 300 < np.median(counts) < 1700
