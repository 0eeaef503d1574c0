"""The seeded generators behind the benchmark workloads and the parity
fixtures (forceatlas2_rc_gb300/graphs.py), on the CPU: reproducible from the
seed, simple undirected edge lists (no self-loops, no repeated pairs, ends in
range), and the shapes the workloads are defined by."""
import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G


def simple(n, a, b):
    assert a.dtype == np.int32 and b.dtype == np.int32
    assert len(a) == len(b)
    if len(a):
        assert a.min() >= 0 and b.min() >= 0 and a.max() < n and b.max() < n
    assert (a != b).all()
    lo, hi = np.minimum(a, b).astype(np.int64), np.maximum(a, b).astype(np.int64)
    assert np.unique(lo * n + hi).size == len(a)


@pytest.mark.parametrize("make", [
    lambda s: G.islands(5, 30, 0.3, 2, seed=s),
    lambda s: G.barabasi_albert(500, 3, seed=s),
    lambda s: G.barabasi_albert_fast(5000, 4, seed=s),
    lambda s: G.pa_test_graph(300, seed=s),
    lambda s: G.sbm(20000, 20, 2.1, 12.0, 2.0, seed=s),
    lambda s: G.erdos_renyi(3000, 8.0, seed=s),
    lambda s: G.island_graph(1000, 10.0, seed=s),
])
def test_generators_are_simple_and_reproducible(make):
    n, a, b = make(3)
    simple(n, a, b)
    n2, a2, b2 = make(3)
    assert n2 == n
    np.testing.assert_array_equal(a, a2)
    np.testing.assert_array_equal(b, b2)
    _, a3, b3 = make(4)
    assert not (np.array_equal(a3, a) and np.array_equal(b3, b))


def test_shapes():
    """Mean degrees near the parameters (after de-duplication); the island
    graph of the README example has 5 islands of 30 nodes; preferential
    attachment makes hubs."""
    n, a, b = G.sbm(100000, 100, 2.1, 12.0, 2.0, seed=1)
    deg = 2.0 * len(a) / n
    assert 11.0 < deg < 14.5
    n, a, b = G.erdos_renyi(50000, 8.0, seed=1)
    assert abs(2.0 * len(a) / n - 8.0) < 0.05
    n, a, b = G.islands(5, 30, 0.3, 2, seed=1)
    assert n == 150
    inside = (a // 30) == (b // 30)
    assert inside.sum() > 0.9 * len(a)
    n, a, b = G.barabasi_albert(2000, 2, seed=1)
    assert len(a) == 2 * (2000 - 2)
    deg = np.bincount(np.concatenate([a, b]), minlength=n)
    assert deg.max() > 10 * deg.mean()


def test_positions():
    p = G.uniform_positions(1000, -50.0, 50.0, seed=7)
    assert p.shape == (1000, 2) and p.dtype == np.float64
    assert p.min() >= -50.0 and p.max() <= 50.0
    np.testing.assert_array_equal(p, G.uniform_positions(1000, -50.0, 50.0, seed=7))
