"""The batched engine (fa2cu_batch_*): many graphs, one persistent launch, one
thread block per graph.

Bars:
  - FP64, graphs of at most 2048 nodes: positions after several iterations
    equal the single-graph device layout's bit for bit (same forces in the
    same order, totals summed serially in node order, the same FP64 speed
    update), in both repulsion modes;
  - FP64, larger graphs: within 1e-9 after 5 iterations (the totals are
    summed in another fixed order);
  - FP32: after one iteration within 1e-4 (norm-wise, relative to the largest
    displacement) of the single-graph FP32 layout;
  - one iteration's forces (fa2cu_batch_forces): FP64 within 1e-12 of the
    oracle's, FP32 within 1e-4 of FP64;
  - a graph's positions are bit-identical alone and in any mix of graphs.
"""
import numpy as np
import pytest

from conftest import rel_err
from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300.batch import Batch, tune
from forceatlas2_rc_gb300.layout import REPULSION_BH, REPULSION_EXACT, Graph, Layout

pytestmark = pytest.mark.gpu


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def case(n, seed, deg=6.0, spread=None):
    """An Erdos-Renyi graph with lognormal weights and float-representable
    start positions."""
    n, a, b = G.erdos_renyi(n, deg, seed=seed)
    w = np.random.default_rng(seed).lognormal(0.0, 0.5, len(a))
    spread = spread or 10.0 * np.sqrt(n)
    pos = f32(G.uniform_positions(n, -spread, spread, seed=seed + 1))
    return Graph(n, a, b, w), pos


SETTINGS = [
    dict(scaling=2.0, gravity=1.0),
    dict(scaling=10.0, gravity=0.5, linlog=True),
    dict(scaling=2.0, gravity=1.0, strong=True),
    dict(scaling=5.0, gravity=1.0, adjust=True),
]


def single(g, pos, prec, exact, iters, **kw):
    rep = REPULSION_EXACT if exact else REPULSION_BH
    with Layout(g, pos, precision=prec, repulsion=rep, **kw) as L:
        L.iterate(iters)
        L.sync()
        return L.positions(), L.speed()


@pytest.mark.parametrize("k", range(len(SETTINGS)))
def test_batch_double_equals_single_graph(gpu, k):
    """FP64 graphs of 40..2000 nodes, exact below 300 nodes: every graph's
    positions and speed after 7 iterations equal the single-graph layout's
    bit for bit."""
    kw = SETTINGS[k]
    sizes = [40, 150, 299, 300, 700, 2000]
    cases = [case(n, 10 * k + i) for i, n in enumerate(sizes)]
    size = [f32(np.random.default_rng(i).uniform(0.5, 3.0, g.n)) for i, (g, _) in
            enumerate(cases)]
    per = [dict(size=s) for s in size]
    with Batch([c[0] for c in cases], [c[1] for c in cases], precision="double",
               exact_below=300, threads=512, per_graph=per, **kw) as B:
        B.iterate(7)
        B.sync()
        got = [(B.positions(i), B.speed(i)) for i in range(len(cases))]
    for i, (g, pos) in enumerate(cases):
        want, sp = single(g, pos, "double", g.n < 300, 7, size=size[i], **kw)
        np.testing.assert_array_equal(got[i][0], want, err_msg=f"graph {i} n={g.n}")
        assert got[i][1]["speed"] == sp["speed"]
        assert got[i][1]["efficiency"] == sp["efficiency"]


def test_batch_double_larger_graphs(gpu):
    """FP64 graphs beyond the serial-totals size: within 1e-9 after 5
    iterations."""
    cases = [case(n, 70 + i) for i, n in enumerate([2049, 6000, 20000])]
    with Batch([c[0] for c in cases], [c[1] for c in cases], precision="double",
               exact_below=0, threads=512, scaling=2.0) as B:
        B.iterate(5)
        B.sync()
        got = [B.positions(i) for i in range(len(cases))]
    for i, (g, pos) in enumerate(cases):
        want, _ = single(g, pos, "double", False, 5, scaling=2.0)
        np.testing.assert_allclose(got[i], want, rtol=1e-9,
                                   atol=1e-9 * np.abs(want).max())


@pytest.mark.parametrize("threads", [256, 512])
def test_batch_single_vs_single_graph(gpu, threads):
    """FP32, one iteration: displacement within 1e-4 of the single-graph FP32
    layout's (exact and Barnes-Hut graphs)."""
    sizes = [60, 500, 1500, 5000, 12000]
    cases = [case(n, 30 + i) for i, n in enumerate(sizes)]
    with Batch([c[0] for c in cases], [c[1] for c in cases], precision="single",
               exact_below=1000, threads=threads, scaling=2.0, linlog=True) as B:
        B.iterate(1)
        B.sync()
        got = [B.positions(i) for i in range(len(cases))]
    for i, (g, pos) in enumerate(cases):
        want, _ = single(g, pos, "single", g.n < 1000, 1, scaling=2.0, linlog=True)
        d_want = want - pos
        err = np.sqrt(((got[i] - want) ** 2).sum(1)).max()
        den = np.sqrt((d_want ** 2).sum(1)).max()
        assert err <= 1e-4 * den, (i, g.n, err / den)


@pytest.mark.parametrize("prec", ["single", "double"])
def test_batch_result_independent_of_mix(gpu, prec):
    """A graph's positions after 20 iterations are bit-identical alone and in
    a batch of 300 other graphs (block size and crossover fixed)."""
    target = [case(3000, 5), case(200, 6)]
    others = [case(int(n), 100 + i) for i, n in enumerate(
        np.random.default_rng(0).integers(2, 4000, 300))]
    args = dict(precision=prec, exact_below=512, threads=512, scaling=2.0,
                gravity=1.0)
    alone = []
    for g, pos in target:
        with Batch([g], [pos], **args) as B:
            B.iterate(20)
            B.sync()
            alone.append(B.positions(0))
    mix = others[:150] + [target[0]] + others[150:] + [target[1]]
    with Batch([c[0] for c in mix], [c[1] for c in mix], **args) as B:
        B.iterate(10)
        B.iterate(10)
        B.sync()
        np.testing.assert_array_equal(B.positions(150), alone[0])
        np.testing.assert_array_equal(B.positions(len(mix) - 1), alone[1])


def test_batch_many_tiny_graphs(gpu):
    """4000 graphs of 1 to 64 nodes (some without edges, some of one node):
    every position stays finite, a lone node only feels gravity (it moves
    towards the origin), and graphs of at least two nodes equal the FP64
    single-graph layout."""
    rng = np.random.default_rng(9)
    cases = []
    for i in range(4000):
        n = int(rng.integers(1, 65))
        if n == 1:
            a = b = np.zeros(0, np.int32)
        else:
            _, a, b = G.erdos_renyi(n, float(rng.uniform(0, 5)), seed=1000 + i)
        pos = f32(G.uniform_positions(n, -20, 20, seed=2000 + i))
        cases.append((Graph(n, a, b, np.ones(len(a))), pos))
    with Batch([c[0] for c in cases], [c[1] for c in cases], precision="double",
               exact_below=65, scaling=2.0, gravity=1.0) as B:
        B.iterate(10)
        B.sync()
        got = [B.positions(i) for i in range(len(cases))]
    for (g, pos), p in zip(cases, got):
        assert np.isfinite(p).all()
        if g.n == 1:
            assert np.hypot(*p[0]) <= np.hypot(*pos[0])
    picks = [i for i, (g, _) in enumerate(cases) if g.n >= 2][:40]
    for i in picks:
        g, pos = cases[i]
        want, _ = single(g, pos, "double", True, 10, scaling=2.0)
        np.testing.assert_array_equal(got[i], want)


def test_batch_fixed_nodes(gpu):
    """Fixed nodes keep their positions; the rest equals the single-graph
    FP64 layout bit for bit."""
    g, pos = case(800, 3)
    fixed = (np.arange(g.n) % 7 == 0).astype(np.int32)
    g2, pos2 = case(400, 4)
    with Batch([g, g2], [pos, pos2], precision="double", exact_below=500,
               threads=512, per_graph=[dict(fixed=fixed), {}], scaling=2.0) as B:
        B.iterate(6)
        B.sync()
        p = B.positions(0)
    np.testing.assert_array_equal(p[fixed == 1], pos[fixed == 1])
    want, _ = single(g, pos, "double", False, 6, fixed=fixed, scaling=2.0)
    np.testing.assert_array_equal(p, want)


def test_batch_tune_and_errors(gpu):
    """The autotuner answers from the allowed values and caches them; invalid
    batches are refused with a message."""
    for prec in ("single", "double"):
        t = tune(0, prec)
        assert t["threads"] in (256, 512)
        assert 64 <= t["exact_below"] <= 32768
        assert t["nodes_per_thread"] in (1, 2)
        assert tune(0, prec) == t
    g, pos = case(100, 1)
    with pytest.raises(RuntimeError, match="threads"):
        Batch([g], [pos], threads=100)
    with pytest.raises(RuntimeError, match="nodes_per_thread"):
        Batch([g], [pos], nodes_per_thread=3)
    bad = Graph(100, [0], [1], [1.0])
    bad.inc_node = np.array([500, 0], np.int32)  # a neighbour out of range
    with pytest.raises(RuntimeError):
        Batch([g, bad], [pos, pos])


@pytest.mark.parametrize("prec", ["single", "double"])
@pytest.mark.parametrize("adjust", [False, True])
def test_batch_exact_tile_shape(gpu, prec, adjust):
    """The exact sum's tile shape (1 or 2 nodes per thread against the
    block's tile of records) changes no bit of a graph's layout: every node
    sums its pairs in ascending order either way. Graphs larger than a block
    of nodes, so that the two-node shape is taken."""
    cases = [case(n, 40 + n % 7) for n in (300, 700, 1500)]
    gs, ps = [c[0] for c in cases], [c[1] for c in cases]
    out = {}
    for npt in (1, 2):
        per = [dict(size=np.full(g.n, 1.5)) for g in gs] if adjust else None
        with Batch(gs, ps, precision=prec, exact_below=1 << 20, threads=256,
                   nodes_per_thread=npt, adjust=adjust, per_graph=per) as B:
            B.iterate(4)
            B.sync()
            out[npt] = [B.positions(i) for i in range(len(gs))]
    for a, b in zip(out[1], out[2]):
        np.testing.assert_array_equal(a, b)


def test_batch_matches_oracle(gpu, orc):
    """Batched FP64 graphs against the oracle directly, not against another
    CUDA path: exact-repulsion graphs after 10 iterations against
    C_forceatlas2 (the oracle's restatement of src/forceatlas2.c) within 1e-9
    (the bar of test-gpu.R:34-58); Barnes-Hut graphs after 1 and after 5
    iterations against the oracle's restatement of the all-GPU pipeline
    (inst/opencl/pipeline.cl in double, FP64 totals) within 1e-9."""
    exact_sizes, bh_sizes = [60, 250, 900], [1500, 3000, 9000]
    raw = []
    for i, n in enumerate(exact_sizes + bh_sizes):
        n, a, b = G.erdos_renyi(n, 6.0, seed=200 + i)
        w = np.random.default_rng(200 + i).lognormal(0.0, 0.5, len(a))
        pos = f32(G.uniform_positions(n, -10 * np.sqrt(n), 10 * np.sqrt(n), seed=300 + i))
        raw.append((n, a, b, w, pos))
    gs = [Graph(n, a, b, w) for n, a, b, w, _ in raw]
    ps = [pos for *_, pos in raw]
    kw = dict(scaling=2.0, gravity=1.0, theta=1.2)
    with Batch(gs, ps, precision="double", exact_below=1000, threads=512, **kw) as B:
        B.iterate(1)
        B.sync()
        one = [B.positions(i) for i in range(len(gs))]
        B.iterate(4)
        B.sync()
        five = [B.positions(i) for i in range(len(gs))]
        B.iterate(5)
        B.sync()
        ten = [B.positions(i) for i in range(len(gs))]

    def close(got, want, what):
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * np.abs(want).max(),
                                   err_msg=what)

    o = orc.Opts(scaling=2.0, gravity=1.0)
    for i in range(len(exact_sizes)):
        n, a, b, w, pos = raw[i]
        close(ten[i], orc.layout(n, a, b, w, pos, None, None, 10, o), f"exact n={n}")
    for i in range(len(exact_sizes), len(raw)):
        n, a, b, w, pos = raw[i]
        go = orc.prepare_large(n, a, b, w)
        for iters, got in ((1, one[i]), (5, five[i])):
            p, keep = orc.full_params(go, iterations=iters, **kw)
            close(got, orc.pipe_run(p, pos, "d"), f"Barnes-Hut n={n}, {iters} iterations")


def test_batch_forces_fp32_vs_fp64_and_oracle(gpu, orc):
    """The forces of one batched iteration (fa2cu_batch_forces) from
    identical positions: FP64 against the oracle's restatement of the
    reference -- C_forceatlas2's exact forces for graphs below the crossover,
    the all-GPU pipeline's Barnes-Hut forces above it -- within 1e-12, and
    FP32 against FP64 within 1e-4 (the per-step force error of config 4)."""
    raw = []
    for i, n in enumerate([60, 400, 1500, 4000]):
        n, a, b = G.erdos_renyi(n, 6.0, seed=400 + i)
        w = np.random.default_rng(400 + i).lognormal(0.0, 0.5, len(a))
        pos = f32(G.uniform_positions(n, -10 * np.sqrt(n), 10 * np.sqrt(n), seed=500 + i))
        raw.append((n, a, b, w, pos))
    gs = [Graph(n, a, b, w) for n, a, b, w, _ in raw]
    ps = [pos for *_, pos in raw]
    got = {}
    for prec in ("single", "double"):
        with Batch(gs, ps, precision=prec, exact_below=1000, threads=512,
                   scaling=2.0, gravity=1.0, theta=1.2) as B:
            B.iterate(1)
            B.sync()
            got[prec] = [B.forces(i) for i in range(len(gs))]
    for i, (n, a, b, w, pos) in enumerate(raw):
        if n < 1000:
            want = orc.forces(n, a, b, w, pos, None, orc.Opts(scaling=2.0, gravity=1.0))
        else:
            go = orc.prepare_large(n, a, b, w)
            p, keep = orc.full_params(go, theta=1.2, scaling=2.0, gravity=1.0)
            want = orc.pipe_forces(p, pos, "d")
        assert rel_err(got["double"][i], want) <= 1e-12, (n, "double")
        assert rel_err(got["single"][i], got["double"][i]) <= 1e-4, (n, "single")
