"""Host-side logic of the serving loop and the MD set-up (no GPU)."""
import collections

import numpy as np

from quip_gb300 import md, serving


def test_admission_is_an_arrival_order_prefix_within_the_share():
    q = collections.deque([("a", 4), ("b", 3), ("c", 5), ("d", 1)])
    batch = serving.admit_prefix(q, lambda r: r[1], 8)
    assert [r[0] for r in batch] == ["a", "b"]          # c would overflow; d must not jump the queue
    assert [r[0] for r in q] == ["c", "d"]


def test_admission_never_starves_a_large_request():
    q = collections.deque([("big", 100), ("small", 1)])
    assert [r[0] for r in serving.admit_prefix(q, lambda r: r[1], 8)] == ["big"]
    assert [r[0] for r in serving.admit_prefix(q, lambda r: r[1], 8)] == ["small"]
    assert serving.admit_prefix(q, lambda r: r[1], 8) == []


def test_poisson_arrivals_rate():
    t = serving.poisson_arrivals(200.0, 20000, seed=3)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 200.0) < 6.0


def test_massconvert_and_maxwell_boltzmann():
    # Units.f95:68 evaluates to 103.6427 (amu -> eV fs^2 / A^2)
    assert abs(md.MASSCONVERT - 103.6427) < 1e-3
    z = np.full(4096, 14)
    v = md.maxwell_boltzmann(z, 1000.0, seed=5)
    m = md.masses(z)
    assert np.allclose((m[:, None] * v).sum(axis=0), 0.0, atol=1e-8)   # zero total momentum
    T = 2 * md.kinetic_energy(v, m) / (3 * len(z) * md.BOLTZMANN_K)
    assert abs(T - 1000.0) < 40.0
