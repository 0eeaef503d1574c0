"""layout_forceatlas2_large / fa2_full_run end to end, restating the
reference's tests/testthat/test-large.R (graphs from this package's seeded
generators instead of igraph's)."""
import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300 import layout_forceatlas2_gpu, layout_forceatlas2_large

pytestmark = pytest.mark.gpu


def pa(n, seed=42):
    n, a, b = G.pa_test_graph(n, seed=seed)
    return n, np.stack([a, b], axis=1)


def start(n, seed=7):
    return G.uniform_positions(n, -50, 50, seed=seed)


def test_theta0_is_exact(gpu, orc):
    """test-large.R:10-38: theta = 0, double, 700 nodes with 30 forced
    coincident (equal Morton codes), 8 option sets: all-GPU == exact CPU
    within 1e-8 after 5 iterations."""
    n, e = pa(700)
    pos = start(n)
    pos[:30] = pos[np.tile(np.arange(3), 10)]
    rng = np.random.default_rng(3)
    w = rng.uniform(0.2, 3.0, len(e))
    size = rng.uniform(0.5, 4.0, n)
    fixed = np.tile([True, False], 350)
    sets = [dict(), dict(scaling_ratio=5.0, gravity=3.0),
            dict(linlog=True, strong_gravity=True),
            dict(dissuade_hubs=True, gravity=0.0),
            dict(weights=w, edge_weight_influence=0.5, jitter_tolerance=0.3),
            dict(prevent_overlap=True, node_size=size),
            dict(prevent_overlap=True, node_size=size, linlog=True,
                 dissuade_hubs=True, weights=w),
            dict(fixed=fixed)]
    for kw in sets:
        got = layout_forceatlas2_large(n, e, 5, init=pos, theta=0.0,
                                       precision="double", **kw)
        ww = kw.get("weights")
        if ww is not None:
            ww = ww ** kw.get("edge_weight_influence", 1.0)
        else:
            ww = np.ones(len(e))
        o = orc.Opts(scaling=kw.get("scaling_ratio", 2.0),
                     gravity=kw.get("gravity", 1.0),
                     jitter_tolerance=kw.get("jitter_tolerance", 1.0),
                     strong=kw.get("strong_gravity", False),
                     linlog=kw.get("linlog", False),
                     outbound=kw.get("dissuade_hubs", False),
                     adjust=kw.get("prevent_overlap", False))
        sz = kw.get("node_size", np.ones(n))
        fx = kw.get("fixed")
        want = orc.layout(n, e[:, 0], e[:, 1], ww, pos, sz,
                          None if fx is None else fx.astype(np.int32), 5, o)
        # the theta = 0 walk adds the same terms as the exact CPU loop but in
        # tree order (1-ulp differences); with prevent_overlap the force is
        # discontinuous at contact (d = 0), which can amplify them
        tol = 1e-5 if kw.get("prevent_overlap") else 1e-8
        np.testing.assert_allclose(got, want, rtol=tol,
                                   atol=tol * np.abs(want).max(),
                                   err_msg=str(list(kw)))


def test_theta_sweep(gpu, orc):
    """test-large.R:40-57: one step on 3000 nodes; the error against the
    exact layout decreases with theta."""
    n, e = pa(3000)
    pos = start(n)
    exact = orc.layout(n, e[:, 0], e[:, 1], np.ones(len(e)), pos, None, None, 1,
                       orc.Opts(scaling=2.0))
    span = exact.max() - exact.min()

    def err(theta, precision="double"):
        xy = layout_forceatlas2_large(n, e, 1, init=pos, theta=theta,
                                      precision=precision)
        return np.abs(xy - exact).max() / span

    assert err(0.1) < 1e-4
    assert err(0.1) < err(0.5) < err(1.2) < 0.02
    assert err(1.2, "single") < 0.02
    assert err(0.0, "single") < 1e-3


def test_reproducible(gpu):
    """test-large.R:59-71: bit-identical reruns."""
    n, e = pa(5000)
    pos = start(n)
    a = layout_forceatlas2_large(n, e, 30, init=pos)
    b = layout_forceatlas2_large(n, e, 30, init=pos)
    np.testing.assert_array_equal(a, b)
    a = layout_forceatlas2_large(n, e, 5, seed=8)
    b = layout_forceatlas2_large(n, e, 5, seed=8)
    np.testing.assert_array_equal(a, b)


def cliques():
    k1 = np.array([(i, j) for i in range(10) for j in range(i + 1, 10)])
    e = np.concatenate([k1, k1 + 10, [[0, 10]]])
    return 20, e


def test_layout_makes_sense(gpu, orc):
    """test-large.R:73-94: two cliques separate; islands keep the edge
    length / sd and sd of the CPU layout within 5 %."""
    n, e = cliques()
    xy = layout_forceatlas2_large(n, e, 500, seed=1)
    d = np.sqrt(((xy[:, None] - xy[None]) ** 2).sum(-1))
    assert np.isfinite(xy).all()
    assert d[:10, :10].max() < d[1:10, 11:20].min()

    rng = np.random.default_rng(5)
    blocks = []
    for k in range(4):
        iu, ju = np.triu_indices(100, 1)
        keep = rng.random(iu.size) < 0.1
        blocks.append(np.stack([iu[keep], ju[keep]], 1) + 100 * k)
    for k in range(4):
        for l in range(k + 1, 4):
            blocks.append(np.stack([rng.integers(0, 100, 2) + 100 * k,
                                    rng.integers(0, 100, 2) + 100 * l], 1))
    e = np.concatenate(blocks)
    n = 400
    pos = start(n)

    def stats(xy):
        el = np.sqrt(((xy[e[:, 0]] - xy[e[:, 1]]) ** 2).sum(1)).mean()
        sd = xy.std(ddof=1)
        return el / sd, sd

    cpu = orc.layout(n, e[:, 0], e[:, 1], np.ones(len(e)), pos, None, None, 300,
                     orc.Opts(scaling=2.0, barnes_hut=False))
    gpu_xy = layout_forceatlas2_large(n, e, 300, init=pos)
    (a1, s1), (a2, s2) = stats(gpu_xy), stats(cpu)
    assert abs(a1 - a2) / a2 < 0.05
    assert abs(s1 - s2) / s2 < 0.05


def test_degenerate(gpu):
    """test-large.R:96-133."""
    assert layout_forceatlas2_large(0, None).shape == (0, 2)
    one = layout_forceatlas2_large(1, None, 10, seed=1)
    assert one.shape == (1, 2) and np.isfinite(one).all()
    for n in range(2, 13):
        ring = np.stack([np.arange(n), (np.arange(n) + 1) % n], 1)
        xy = layout_forceatlas2_large(n, ring, 50, seed=n)
        assert np.isfinite(xy).all()
        d = np.sqrt(((xy[:, None] - xy[None]) ** 2).sum(-1))
        assert d[~np.eye(n, dtype=bool)].min() > 0
    assert np.isfinite(layout_forceatlas2_large(300, None, 100, seed=1)).all()
    e = np.array([[0, 0], [0, 1], [0, 1], [1, 2]])
    assert np.isfinite(layout_forceatlas2_large(5, e, 100, seed=1)).all()
    n, e = pa(500)
    zero = np.zeros((n, 2))
    np.testing.assert_array_equal(layout_forceatlas2_large(n, e, 20, init=zero), zero)
    line = np.stack([np.arange(1.0, 501.0), np.zeros(500)], 1)
    assert np.isfinite(layout_forceatlas2_large(n, e, 20, init=line)).all()
    pos = start(n)
    pos[:300] = 1.0
    assert np.isfinite(layout_forceatlas2_large(n, e, 20, init=pos)).all()
    np.testing.assert_allclose(layout_forceatlas2_large(n, e, 0, init=pos), pos,
                               rtol=1e-6)


def test_api_errors(gpu):
    n, e = pa(60)
    from forceatlas2_rc_gb300 import gpu_devices
    nd = len(gpu_devices())
    with pytest.raises(ValueError, match="device"):
        layout_forceatlas2_large(n, e, 20, device=nd + 1)
    with pytest.raises(ValueError, match="device"):
        layout_forceatlas2_large(n, e, 20, device=0)
    with pytest.raises(ValueError, match="theta"):
        layout_forceatlas2_large(n, e, 20, theta=-1)
    with pytest.raises(ValueError, match="arg"):
        layout_forceatlas2_gpu(n, e, 20, precision="half")


def test_timings(gpu):
    n, e = pa(2000)
    xy, t = layout_forceatlas2_large(n, e, 20, seed=1, timings=True)
    assert list(t) == ["total", "codes", "sort", "tree", "repulsion",
                       "attraction", "move"]
    assert all(v >= 0 for v in t.values()) and t["repulsion"] > 0
    assert t["total"] >= sum(t[k] for k in list(t)[1:]) * 0.5


def test_gpu_layout_double_equals_cpu(gpu, orc):
    """test-gpu.R:34-58 restated for the all-device layout_forceatlas2_gpu:
    exact repulsion in double == the CPU layout within 1e-9."""
    n, e = pa(400)
    pos = start(n)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.2, 3.0, len(e))
    size = rng.uniform(0.5, 4.0, n)
    sets = [dict(), dict(scaling_ratio=5.0, gravity=3.0),
            dict(linlog=True, dissuade_hubs=True, strong_gravity=True),
            dict(weights=w, edge_weight_influence=0.5),
            dict(prevent_overlap=True, node_size=size),
            dict(fixed=np.tile([True, False], 200))]
    for kw in sets:
        got = layout_forceatlas2_gpu(n, e, 10, init=pos, barnes_hut=False,
                                     precision="double", **kw)
        ww = kw.get("weights")
        ww = np.ones(len(e)) if ww is None else ww ** kw.get("edge_weight_influence", 1.0)
        o = orc.Opts(scaling=kw.get("scaling_ratio", 2.0),
                     gravity=kw.get("gravity", 1.0),
                     strong=kw.get("strong_gravity", False),
                     linlog=kw.get("linlog", False),
                     outbound=kw.get("dissuade_hubs", False),
                     adjust=kw.get("prevent_overlap", False))
        fx = kw.get("fixed")
        want = orc.layout(n, e[:, 0], e[:, 1], ww, pos, kw.get("node_size"),
                          None if fx is None else fx.astype(np.int32), 10, o)
        np.testing.assert_allclose(got, want, rtol=1e-9,
                                   atol=1e-9 * np.abs(want).max(),
                                   err_msg=str(list(kw)))


def test_gpu_layout_single_close_to_cpu(gpu, orc):
    """test-gpu.R:60-79: single precision stays within 1e-3 after 2
    iterations, and is not identical."""
    n, e = pa(400)
    pos = start(n)
    cpu = orc.layout(n, e[:, 0], e[:, 1], np.ones(len(e)), pos, None, None, 2,
                     orc.Opts(scaling=2.0))
    got = layout_forceatlas2_gpu(n, e, 2, init=pos, barnes_hut=False)
    assert np.abs(got - cpu).max() / (cpu.max() - cpu.min()) < 1e-3
    assert not np.array_equal(got, cpu)


def layout_stats(xy, a, b, k=10):
    """Scale-free statistics of a final layout: mean edge length over the
    sd of the coordinates, and neighbourhood preservation -- per node, the
    share of its graph neighbours among its k nearest nodes in the plane
    (up to min(k, degree)), averaged over the nodes with neighbours."""
    el = np.sqrt(((xy[a] - xy[b]) ** 2).sum(1)).mean() / xy.std(ddof=1)
    from scipy.spatial import cKDTree
    n = len(xy)
    _, nn = cKDTree(xy).query(xy, k + 1)
    nbr = [set() for _ in range(n)]
    for u, v in zip(a, b):
        nbr[u].add(v)
        nbr[v].add(u)
    pres = [len(nbr[i] & set(nn[i, 1:])) / min(k, len(nbr[i]))
            for i in range(n) if nbr[i]]
    return el, float(np.mean(pres))


@pytest.mark.parametrize("precision", ["single", "double"])
def test_layout_statistics_seed_averaged(gpu, orc, precision):
    """Final layouts, whose trajectories diverge chaotically, are compared by
    seed-averaged statistics: a 3000-node stochastic block model (30 blocks
    of power-law sizes, lognormal weights), 300 iterations of Barnes-Hut
    (theta 1.2) on the device against the reference's CPU engine (quadtree
    Barnes-Hut), over four seeds: normalised edge length within 5 %,
    neighbourhood preservation within 0.03 (both near 0.38 and 0.13 here)."""
    n, a, b = G.sbm(3000, 30, 2.1, 12.0, 1.0, seed=11)
    w = np.random.default_rng(3).lognormal(0.0, 0.5, len(a))
    edges = np.stack([a, b], 1)
    r = 10.0 * np.sqrt(n)
    gs, cs = [], []
    for seed in range(4):
        pos = G.uniform_positions(n, -r, r, seed=100 + seed)
        xy = layout_forceatlas2_large(n, edges, 300, weights=w, init=pos,
                                      precision=precision, theta=1.2)
        cpu = orc.layout(n, a, b, w, pos, None, None, 300,
                         orc.Opts(scaling=2.0, barnes_hut=True, theta=1.2, threads=8))
        gs.append(layout_stats(xy, a, b))
        cs.append(layout_stats(cpu, a, b))
    g_el, g_np = np.mean(gs, axis=0)
    c_el, c_np = np.mean(cs, axis=0)
    assert abs(g_el - c_el) / c_el < 0.05, (g_el, c_el)
    assert abs(g_np - c_np) < 0.03, (g_np, c_np)
