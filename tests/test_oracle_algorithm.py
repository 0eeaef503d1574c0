"""The reference's algorithm tests (tests/testthat/test-algorithm.R) restated
for the C oracle, on the CPU: the oracle against an independent numpy
transcription of Gephi's iteration (tests/gephi_numpy.py, restating
helper-reference.R), Barnes-Hut against the exact sum, thread invariance,
layout sanity, fixed nodes and degenerate graphs. Graphs come from this
package's seeded generators (igraph's streams cannot be reproduced), with
the reference tests' sizes and options."""
import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G
from gephi_numpy import gephi_layout, mean_rel


def pa(n, seed=42):
    n, a, b = G.pa_test_graph(n, seed=seed)
    return n, a, b


def start(n, seed=7):
    return G.uniform_positions(n, -50.0, 50.0, seed=seed)


def run(orc, n, a, b, pos, iterations, w=None, size=None, fixed=None, **kw):
    kw.setdefault("scaling", 10.0)
    w = np.ones(len(a)) if w is None else w
    return orc.layout(n, a, b, w, pos, size, fixed, iterations, orc.Opts(**kw))


def random_init(n, seed):
    r = 10.0 * np.sqrt(n)
    return np.random.default_rng(seed).uniform(-r, r, (n, 2))


def test_oracle_agrees_with_gephi_transcription(orc):
    """test-algorithm.R:1-17: 10 iterations at 1e-9, 100 at 1e-3."""
    n, a, b = pa(40)
    pos = start(n)
    assert mean_rel(run(orc, n, a, b, pos, 10),
                    gephi_layout(n, a, b, pos, 10, scaling=10.0)) < 1e-9
    assert mean_rel(run(orc, n, a, b, pos, 100),
                    gephi_layout(n, a, b, pos, 100, scaling=10.0)) < 1e-3


def test_every_option_agrees_with_gephi_transcription(orc):
    """test-algorithm.R:19-61, tolerance 1e-8 after 10 iterations.
    edge_weight_influence 0.5 reaches the C code as the square roots of the
    weights."""
    n, a, b = pa(40)
    pos = start(n)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.2, 3.0, len(a))
    size = rng.uniform(0.5, 4.0, n)
    cases = [
        (dict(strong=True, gravity=0.3), dict(strong=True, gravity=0.3), None, None),
        (dict(linlog=True, scaling=3.0), dict(linlog=True, scaling=3.0), None, None),
        (dict(outbound=True, gravity=0.0), dict(outbound=True, gravity=0.0), None, None),
        (dict(jitter_tolerance=0.2), dict(jt_user=0.2), np.sqrt(w), None),
        (dict(adjust=True), dict(adjust=True), None, size),
        (dict(adjust=True, linlog=True, outbound=True),
         dict(adjust=True, linlog=True, outbound=True), w, size),
    ]
    for ok, gk, ww, sz in cases:
        got = run(orc, n, a, b, pos, 10, w=ww, size=sz, **ok)
        gk = dict(gk)
        gk.setdefault("scaling", 10.0)
        want = gephi_layout(n, a, b, pos, 10, w=ww,
                            size=1.0 if sz is None else sz, **gk)
        assert mean_rel(got, want) < 1e-8, ok


def test_barnes_hut_converges_to_exact(orc):
    """test-algorithm.R:63-86: theta = 0 equals the exact sum (also with
    prevent_overlap); the error of one step grows with theta and stays
    below 1e-4 at 0.1 and 0.02 at 1.2."""
    n, a, b = pa(300)
    pos = start(n)
    assert mean_rel(run(orc, n, a, b, pos, 5, barnes_hut=True, theta=0.0),
                    run(orc, n, a, b, pos, 5)) < 1e-9
    size = np.full(n, 2.0)
    assert mean_rel(
        run(orc, n, a, b, pos, 3, size=size, barnes_hut=True, theta=0.0, adjust=True),
        run(orc, n, a, b, pos, 3, size=size, adjust=True)) < 1e-9
    exact = run(orc, n, a, b, pos, 1)
    span = exact.max() - exact.min()

    def err(theta):
        got = run(orc, n, a, b, pos, 1, barnes_hut=True, theta=theta)
        return np.abs(got - exact).max() / span

    e01, e05, e12 = err(0.1), err(0.5), err(1.2)
    assert e01 < 1e-4
    assert e01 < e05 < e12
    assert e12 < 0.02


@pytest.mark.parametrize("bh", [False, True])
def test_threads_do_not_change_the_result(orc, bh):
    """test-algorithm.R:88-103: bit-identical for 1 and 2 threads."""
    n, a, b = pa(500)
    pos = start(n)
    np.testing.assert_array_equal(
        run(orc, n, a, b, pos, 40, barnes_hut=bh, threads=1),
        run(orc, n, a, b, pos, 40, barnes_hut=bh, threads=2))
    if not bh:
        np.testing.assert_array_equal(
            run(orc, n, a, b, pos, 40, adjust=True, threads=1),
            run(orc, n, a, b, pos, 40, adjust=True, threads=2))


def two_cliques():
    a, b = [], []
    for base in (0, 10):
        for i in range(10):
            for j in range(i + 1, 10):
                a.append(base + i)
                b.append(base + j)
    a.append(0)
    b.append(10)
    return 20, np.array(a, np.int32), np.array(b, np.int32)


def pairwise(xy):
    d = xy[:, None, :] - xy[None, :, :]
    return np.sqrt((d ** 2).sum(axis=2))


def test_the_layout_makes_sense(orc):
    """test-algorithm.R:115-147 with the R function's defaults (scaling 2,
    gravity 1, exact below 1000 nodes): two cliques joined by one edge end
    up apart; a converged layout barely moves; more repulsion spreads the
    layout, more gravity (or strong gravity) shrinks it."""
    n, a, b = two_cliques()
    pos = random_init(n, 1)
    xy = run(orc, n, a, b, pos, 500, scaling=2.0)
    d = pairwise(xy)
    assert np.isfinite(xy).all()
    assert d[:10, :10].max() < d[1:10, 11:20].min()
    again = run(orc, n, a, b, xy, 50, scaling=2.0)
    assert np.abs(again - xy).max() / (xy.max() - xy.min()) < 0.01

    def spread(**kw):
        kw.setdefault("scaling", 2.0)
        dd = pairwise(run(orc, n, a, b, pos, 500, **kw))
        return dd[np.triu_indices(n, 1)].mean()

    assert spread(scaling=50.0) > spread(scaling=5.0)
    assert spread(gravity=20.0) < spread(gravity=1.0)
    assert spread(strong=True) < spread()


def test_prevent_overlap_separates_nodes(orc):
    """test-algorithm.R:128-137: a 30-clique packs closer than 12; with
    prevent_overlap and radius 6 it ends with every pair >= 12 apart."""
    n = 30
    iu = np.triu_indices(n, 1)
    a, b = iu[0].astype(np.int32), iu[1].astype(np.int32)
    xy = run(orc, n, a, b, random_init(n, 2), 500, scaling=1.0)
    assert pairwise(xy)[iu].min() < 12
    xy2 = run(orc, n, a, b, xy, 500, scaling=1.0, adjust=True, size=np.full(n, 6.0))
    assert pairwise(xy2)[iu].min() >= 12


def test_fixed_nodes_do_not_move(orc):
    """test-algorithm.R:149-160."""
    n, a, b = pa(30)
    pos = start(n)
    fixed = np.zeros(n, np.int32)
    fixed[:5] = 1
    xy = run(orc, n, a, b, pos, 100, fixed=fixed)
    np.testing.assert_array_equal(xy[:5], pos[:5])
    assert (xy[5:] != pos[5:]).all()
    assert mean_rel(run(orc, n, a, b, pos, 10, fixed=fixed),
                    gephi_layout(n, a, b, pos, 10, scaling=10.0,
                                 fixed=fixed.astype(bool))) < 1e-9


def test_degenerate_graphs(orc):
    """test-algorithm.R:162-194: one node; no edges; self-loops and
    multi-edges; all nodes at one place (nothing moves); coincident nodes
    with theta = 0 equal the exact sum; zero iterations."""
    one = run(orc, 1, np.zeros(0, np.int32), np.zeros(0, np.int32), random_init(1, 1), 100)
    assert one.shape == (1, 2) and np.isfinite(one).all()
    e = np.zeros(0, np.int32)
    assert np.isfinite(run(orc, 20, e, e, random_init(20, 1), 2000, scaling=2.0)).all()
    la = np.array([0, 0, 0, 1], np.int32)
    lb = np.array([0, 1, 1, 2], np.int32)
    for bh in (False, True):
        assert np.isfinite(run(orc, 5, la, lb, random_init(5, 1), 200,
                               scaling=2.0, barnes_hut=bh)).all()
    n, a, b = pa(50)
    zero = np.zeros((n, 2))
    for bh in (False, True):
        np.testing.assert_array_equal(run(orc, n, a, b, zero, 2000, barnes_hut=bh), zero)
    pos = start(n)
    pos[:20] = 1.0
    assert mean_rel(run(orc, n, a, b, pos, 5, barnes_hut=True, theta=0.0),
                    run(orc, n, a, b, pos, 5)) < 1e-9
    assert np.isfinite(run(orc, n, a, b, pos, 30, barnes_hut=True)).all()
    np.testing.assert_array_equal(run(orc, n, a, b, pos, 0), pos)


def test_self_loops_and_multi_edges_in_the_transcription(orc):
    """Masses count every edge end (a self-loop twice, a repeated edge each
    time, reference src/forceatlas2.c:592-603); the oracle and the numpy
    transcription agree on such a graph with every option that reads the
    masses."""
    la = np.array([0, 0, 0, 1, 3, 4, 4], np.int32)
    lb = np.array([0, 1, 1, 2, 4, 3, 4], np.int32)
    pos = start(6, seed=11)
    np.testing.assert_array_equal(orc.mass(6, la, lb)[0], [5, 4, 2, 3, 5, 1])
    for kw in (dict(), dict(outbound=True), dict(linlog=True), dict(strong=True)):
        assert mean_rel(run(orc, 6, la, lb, pos, 10, **kw),
                        gephi_layout(6, la, lb, pos, 10, scaling=10.0, **kw)) < 1e-9, kw
