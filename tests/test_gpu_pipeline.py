"""The all-GPU pipeline (Morton codes, radix sort, Karras tree, bottom-up
centres of mass, stackless Barnes-Hut, attraction, swing, apply) against the
oracle and the golden fixtures of the reference.

Bars: Morton keys, sorted order (ties by index) and the tree's child /
range / parent arrays bit-exact in both precisions against the same
construction; per-step forces within 1e-12 (double) of the oracle, and within
1e-4 (single, norm-wise relative) of the double-precision forces from
identical positions (coordinates representable in float; 2e-3 with
prevent_overlap, whose near-contact force is ill-conditioned in float).

The single-precision path builds its tree with the reference's *double*
construction over the float positions (keys, order and the regions' sums in
double, records rounded to float), and settles opening tests within 1e-4 of
the boundary in double: both paths approximate the same regions.
"""
import numpy as np
import pytest

from conftest import rel_err
from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300.layout import REPULSION_BH, REPULSION_EXACT, Graph, Layout

pytestmark = pytest.mark.gpu

PREC = {"f": "single", "d": "double"}


def f32(a):
    """Values the single-precision path represents exactly."""
    return np.asarray(a).astype(np.float32).astype(np.float64)


def assert_ni_single(got, want_double):
    """FP32 region records: centre of mass from float-float sums, size^2 from
    the float bounding box -- within a few float ulps of the double
    construction (1 ulp = 6e-8 relative)."""
    want = np.asarray(want_double)
    scale = np.abs(want[:, :2]).max() if want.size else 1.0
    np.testing.assert_allclose(got[:, :2], want[:, :2], rtol=3e-7, atol=3e-7 * scale)
    np.testing.assert_allclose(got[:, 2], want[:, 2], rtol=1e-7)
    np.testing.assert_allclose(got[:, 3], want[:, 3], rtol=1e-6)


def make_layout(n, a, b, w, pos, precision="single", repulsion=REPULSION_BH,
                outbound=False, **kw):
    g = Graph(n, a, b, w, outbound=outbound)
    return Layout(g, pos, precision=precision, repulsion=repulsion, **kw)


def tree_cases(golden):
    g = golden
    yield "pb", g["pb_pos"], g["pb_mass"]
    yield "pl", np.stack([np.arange(64.0), np.zeros(64)], 1), np.ones(64)
    yield "p2", np.array([[0.0, 0.0], [1.0, 1.0]]), np.ones(2)


def test_tree_bit_exact_golden_double(gpu, golden):
    """FP64: keys, order, child, range, parent and the regions' (cx, cy, m,
    size^2) equal the reference's pipeline.cl (double) run on the CPU."""
    for tag, pos, m in tree_cases(golden):
        n = len(pos)
        a = np.zeros(0, np.int32)
        g = Graph(n, a, a, np.zeros(0))
        g.mass = np.ascontiguousarray(m, dtype=np.float64)
        with Layout(g, pos, precision="double") as L:
            t = L.tree(pos)
        for k in ("key", "order", "child", "range", "parent", "ni"):
            np.testing.assert_array_equal(t[k], golden[f"{tag}_d_{k}"],
                                          err_msg=f"{tag} {k}")


def test_tree_bit_exact_golden_single(gpu, golden):
    """FP32: the tree is the reference's double construction over the
    float-rounded positions (tests/golden pb32); region records are those
    values rounded to float."""
    pos, m = golden["pb32_pos"], golden["pb_mass"]
    n = len(pos)
    a = np.zeros(0, np.int32)
    g = Graph(n, a, a, np.zeros(0))
    g.mass = np.ascontiguousarray(m, dtype=np.float64)
    with Layout(g, pos, precision="single") as L:
        t = L.tree(pos)
    for k in ("key", "order", "child", "range", "parent"):
        np.testing.assert_array_equal(t[k], golden[f"pb32_d_{k}"], err_msg=k)
    assert_ni_single(t["ni"], golden["pb32_d_ni"])


@pytest.mark.parametrize("prec", ["f", "d"])
@pytest.mark.parametrize("n,dup", [(5000, 500), (70000, 0), (3, 3)])
def test_tree_bit_exact_oracle(gpu, orc, prec, n, dup):
    rng = np.random.default_rng(n)
    pos = rng.uniform(-1e3, 1e3, size=(n, 2))
    if dup:
        pos[:dup] = pos[rng.integers(0, min(7, n), dup)]
    if prec == "f":
        pos = f32(pos)
    m = rng.integers(1, 20, n).astype(float)
    a = np.zeros(0, np.int32)
    g = Graph(n, a, a, np.zeros(0))
    g.mass = m
    with Layout(g, pos, precision=PREC[prec]) as L:
        t = L.tree(pos)
    r = orc.pipe_build(n, pos, m, "d")
    for k in ("key", "order", "child", "range", "parent"):
        np.testing.assert_array_equal(t[k], r[k], err_msg=k)
    if prec == "d":
        np.testing.assert_array_equal(t["ni"], r["ni"])
    else:
        assert_ni_single(t["ni"], r["ni"])


@pytest.mark.parametrize("span", [2e3, 7.3, 3e6])
def test_morton_keys_at_cell_boundaries(gpu, orc, span):
    """FP32 Morton keys (float-float quantisation, double fallback near a
    cell boundary) equal the double construction's for float positions placed
    within a few ulps of the quantisation boundaries (v - min) * scale = k,
    at three extents."""
    rng = np.random.default_rng(int(span))
    n = 60000
    lo = -0.37 * span
    scale = 65535.0 / span
    k = rng.integers(0, 65536, size=(n, 2)).astype(np.float64)
    pos = lo + k / scale
    pos = np.nextafter(pos.astype(np.float32),
                       np.where(rng.random((n, 2)) < 0.5, -np.inf, np.inf).astype(np.float32))
    pos = pos.astype(np.float64)
    pos[:3] = [[lo, lo], [lo + span, lo + span], [lo + span / 2, lo]]  # the extent
    pos = f32(pos)
    m = np.ones(n)
    a = np.zeros(0, np.int32)
    g = Graph(n, a, a, np.zeros(0))
    g.mass = m
    with Layout(g, pos, precision="single") as L:
        t = L.tree(pos)
    r = orc.pipe_build(n, pos, m, "d")
    np.testing.assert_array_equal(t["key"], r["key"])
    np.testing.assert_array_equal(t["order"], r["order"])


def morton_np(pos):
    """Morton keys of the double construction (pipeline.cl:105-130) in numpy:
    IEEE double subtraction and product, clamp, truncate, interleave."""
    mn = pos.min(axis=0)
    ext = max(pos[:, 0].max() - mn[0], pos[:, 1].max() - mn[1])
    scale = 65535.0 / ext if ext > 0 else 0.0
    q = np.clip((pos - mn) * scale, 0.0, 65535.0).astype(np.uint32)

    def spread(v):
        v = v.astype(np.uint64)
        v = (v | (v << 8)) & 0x00FF00FF
        v = (v | (v << 4)) & 0x0F0F0F0F
        v = (v | (v << 2)) & 0x33333333
        v = (v | (v << 1)) & 0x55555555
        return v
    return (spread(q[:, 0]) | (spread(q[:, 1]) << 1)).astype(np.uint32)


@pytest.mark.parametrize("prec", ["single", "double"])
def test_sort_large_with_ties(gpu, prec):
    """3,000,000 nodes, a third of them on 1000 shared positions: the device
    keys and order equal numpy's keys and stable argsort (ties by index)."""
    rng = np.random.default_rng(17)
    n = 3_000_000
    pos = rng.uniform(-5e3, 5e3, size=(n, 2))
    dup = rng.random(n) < 0.33
    pos[dup] = pos[rng.integers(0, 1000, dup.sum())]
    if prec == "single":
        pos = f32(pos)
    a = np.zeros(0, np.int32)
    g = Graph(n, a, a, np.zeros(0))
    with Layout(g, pos, precision=prec) as L:
        t = L.tree(pos)
    key = morton_np(pos)
    order = np.argsort(key, kind="stable")
    np.testing.assert_array_equal(t["order"], order)
    np.testing.assert_array_equal(t["key"], key[order])


PIPE_SETS = [dict(), dict(linlog=True, adjust=True, theta=0.5),
             dict(strong=True, theta=0.0), dict(outbound=True, gravity=0.0)]


def _pipe_case(golden):
    g = golden
    return g["pb_pos"], g["pb_from"], g["pb_to"], g["pf_w"], g["pf_size"]


@pytest.mark.parametrize("k", range(len(PIPE_SETS)))
def test_pipeline_forces_double_vs_golden(gpu, golden, k):
    """FP64 per-step forces of the Barnes-Hut pipeline: <= 1e-12 against the
    reference's own pipeline.cl (double) on the CPU."""
    pos, a, b, w, s = _pipe_case(golden)
    n = len(pos)
    d = dict(PIPE_SETS[k])
    ob = d.pop("outbound", False)
    with make_layout(n, a, b, w, pos, "double", outbound=ob, size=s, **d) as L:
        f = L.forces(pos)
    want = golden[f"pf_{k}_d"]
    assert rel_err(f, want) <= 1e-12


@pytest.mark.parametrize("k", range(len(PIPE_SETS)))
def test_pipeline_forces_single(gpu, golden, orc, k):
    """FP32 per-step forces: close to the oracle's computation of the same
    path, and within 1e-4 of the double-precision forces from identical
    positions. (The golden case puts nodes at the same place on purpose;
    there the double construction's own centre-of-mass rounding yields huge
    forces, as the reference's does, so fresh positions are used.)"""
    pos, a, b, w, s = _pipe_case(golden)
    n = len(pos)
    d = dict(PIPE_SETS[k])
    ob = d.pop("outbound", False)
    pos2 = f32(G.uniform_positions(n, -50, 50, seed=11))
    s2 = f32(s)
    gr = orc.prepare_large(n, a, b, w, outbound=ob)
    p, keep = orc.full_params(gr, size=s2, **d)
    with make_layout(n, a, b, w, pos2, "single", outbound=ob, size=s2, **d) as L:
        f = L.forces(pos2)
    assert rel_err(f, orc.pipe_forces(p, pos2, "m")) <= 1e-5
    assert rel_err(f, orc.pipe_forces(p, pos2, "d")) <= (2e-3 if d.get("adjust") else 1e-4)


@pytest.mark.parametrize("theta", [0.0, 0.5, 1.2])
def test_pipeline_forces_larger(gpu, orc, theta):
    """BA graph of 20000 nodes with lognormal weights: double == oracle
    (<= 1e-12); single vs double <= 1e-4."""
    n, a, b = G.barabasi_albert(20000, 3, seed=2)
    w = np.random.default_rng(1).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0, 1000, seed=3))
    go = orc.prepare_large(n, a, b, w)
    p, keep = orc.full_params(go, theta=theta, scaling=2.0)
    want_d = orc.pipe_forces(p, pos, "d")
    with make_layout(n, a, b, w, pos, "double", theta=theta) as L:
        fd = L.forces(pos)
    assert rel_err(fd, want_d) <= 1e-12
    with make_layout(n, a, b, w, pos, "single", theta=theta) as L:
        ff = L.forces(pos)
    assert rel_err(ff, orc.pipe_forces(p, pos, "m")) <= 1e-5
    assert rel_err(ff, want_d) <= 1e-5  # measured ~1e-6: same tree, same decisions


def test_exact_forces_match_forceatlas2c(gpu, golden):
    """Exact repulsion + gravity + attraction (FP64) reproduce the
    reference's recorded per-step forces of src/forceatlas2.c."""
    from golden.make_golden import OPTION_SETS
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    for k, d in enumerate(OPTION_SETS):
        d = dict(d)
        kw = dict(scaling=d.pop("scaling", 10.0), gravity=d.pop("gravity", 1.0),
                  strong=d.pop("strong", False), linlog=d.pop("linlog", False),
                  adjust=d.pop("adjust", False))
        ob = d.pop("outbound", False)
        with make_layout(n, a, b, w, pos, "double", REPULSION_EXACT,
                         outbound=ob, size=size, **kw) as L:
            f = L.forces(pos)
        err = rel_err(f, g[f"cf_{k}_0_None"])
        assert err <= 1e-12, (k, err)


def test_config1_per_step_gate(gpu, orc):
    """Islands 5 x 30, exact, FP64, scaling 2, gravity 1, 1000 iterations:
    at every step, the GPU forces at the oracle's positions are within
    1e-12 of src/forceatlas2.c's."""
    n, a, b = G.islands(5, 30, 0.3, 2, seed=1)
    w = np.ones(len(a))
    pos0 = G.uniform_positions(n, 0.0, 1.0, seed=1)
    o = orc.Opts(scaling=2.0, gravity=1.0)
    trace = orc.layout_trace(n, a, b, w, pos0, None, None, 1000, o)
    worst = 0.0
    with make_layout(n, a, b, w, pos0, "double", REPULSION_EXACT, scaling=2.0) as L:
        for t in range(0, 1001):
            f = L.forces(trace[t])
            want = orc.forces(n, a, b, w, trace[t], None, o)
            worst = max(worst, rel_err(f, want))
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("k", range(6))
def test_exact_trajectory_double(gpu, golden, k):
    """10 iterations of the exact GPU layout in double == C_forceatlas2
    (tolerance 1e-9 as test-gpu.R:34-58)."""
    from golden.make_golden import OPTION_SETS
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    d = dict(OPTION_SETS[k])
    kw = dict(scaling=d.pop("scaling", 10.0), gravity=d.pop("gravity", 1.0),
              strong=d.pop("strong", False), linlog=d.pop("linlog", False),
              adjust=d.pop("adjust", False))
    ob = d.pop("outbound", False)
    with make_layout(n, a, b, w, pos, "double", REPULSION_EXACT, outbound=ob,
                     size=size, **kw) as L:
        L.iterate(10)
        L.sync()
        xy = L.positions()
    want = g[f"cl_{k}_0"]
    np.testing.assert_allclose(xy, want, rtol=1e-9, atol=1e-9 * np.abs(want).max())


def test_fixed_nodes(gpu, golden):
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    fixed = g["cl_fixed_mask"]
    with make_layout(n, a, b, w, pos, "double", REPULSION_EXACT, scaling=10.0,
                     fixed=fixed) as L:
        L.iterate(10)
        L.sync()
        xy = L.positions()
    np.testing.assert_array_equal(xy[fixed == 1], pos[fixed == 1])
    np.testing.assert_allclose(xy, g["cl_fixed"], rtol=1e-9,
                               atol=1e-9 * np.abs(g["cl_fixed"]).max())


@pytest.mark.parametrize("prec", ["single", "double"])
@pytest.mark.parametrize("adjust", [False, True])
def test_warp_walk_equals_thread_walk(gpu, prec, adjust):
    """Every walk computes the interactions of one independent walk per
    thread. The warp-synchronous walk (lanes keep their own decisions), the
    per-thread walk without its register bound and the walks of two or four
    nodes per thread add them up in the same order: forces identical to the
    per-thread walk (the warp walk in float within 1e-6: its far-field loads
    are shared). The deferred walk (the FP32 default) sums the far regions
    first, then the queued node pairs: within 1e-6 in float, 1e-12 in
    double, and reproducible."""
    n, a, b = G.barabasi_albert(30000, 3, seed=4)
    w = np.random.default_rng(2).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, -2000, 2000, seed=5))
    pos[:40] = pos[np.tile(np.arange(4), 10)]  # coincident nodes
    size = f32(np.random.default_rng(3).uniform(0.5, 4.0, n))
    got = {}
    with make_layout(n, a, b, w, pos, prec, size=size, adjust=adjust,
                     theta=1.2) as L:
        got["default"] = L.forces(pos)
        for name, mode in (("warp", 0), ("thread", 1), ("wide", 2), ("pair", 3),
                           ("quad", 4), ("deferred", 5), ("thread2", 1), ("deferred2", 5)):
            L.option("walk", mode)
            got[name] = L.forces(pos)
    ft = got["thread"]
    for k in ("thread2", "wide", "pair", "quad"):
        np.testing.assert_array_equal(got[k], ft, err_msg=k)
    np.testing.assert_array_equal(got["deferred2"], got["deferred"])
    np.testing.assert_array_equal(got["default"],
                                  got["deferred"] if prec == "single" else ft)
    if prec == "double":
        np.testing.assert_array_equal(got["warp"], ft)
        assert rel_err(got["deferred"], ft) <= 1e-12
    else:
        assert rel_err(got["warp"], ft) <= 1e-6
        assert rel_err(got["deferred"], ft) <= 1e-6


@pytest.mark.parametrize("prec", ["single", "double"])
def test_climb_leaves_per_thread_give_the_same_tree(gpu, prec):
    """The tree's sums are the same whichever thread completes a region: 1,
    2, 4 or 8 leaves per climbing thread (contiguous or interleaved over the
    warp) give the same regions, hence bit-identical forces and
    trajectories, on a graph with coincident nodes."""
    n, a, b = G.barabasi_albert(30000, 3, seed=6)
    w = np.ones(len(a))
    pos = f32(G.uniform_positions(n, -2000, 2000, seed=7))
    pos[:64] = pos[np.tile(np.arange(8), 8)]
    want_f = None
    for mode in (1, 2, 4, 8, -2, -4):
        with make_layout(n, a, b, w, pos, prec, theta=1.2) as L:
            L.option("climb", mode)
            f = L.forces(pos)
            L.iterate(5)
            L.sync()
            xy = L.positions()
        if want_f is None:
            want_f, want_xy = f, xy
        np.testing.assert_array_equal(f, want_f, err_msg=f"climb {mode}")
        np.testing.assert_array_equal(xy, want_xy, err_msg=f"climb {mode}")


@pytest.mark.parametrize("prec,n", [("single", 200_000), ("single", 3000),
                                    ("double", 50_000), ("double", 1500)])
def test_totals_are_fp64_compensated(gpu, prec, n):
    """The swing/traction totals that drive the speed controller are summed
    in FP64 with compensation in both paths (float-float within a warp in
    FP32, whose 48 bits hold a warp's sum): they equal the exact sum
    (math.fsum) of the same per-node values, fixed nodes excluded, within
    1e-12 relative (reference src/forceatlas2.c:758-777)."""
    import math
    n, a, b = G.barabasi_albert(n, 3, seed=8)
    w = np.random.default_rng(4).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0, 1000, seed=9))
    fixed = (np.random.default_rng(5).random(n) < 0.05).astype(np.int32)
    with make_layout(n, a, b, w, pos, prec, theta=1.2, fixed=fixed) as L:
        L.option("keep_traction", 1)
        L.iterate(3)
        L.sync()
        sw, tr = L.swing(traction=True)
        st = L.speed()
    keep = fixed == 0
    for got, vals in ((st["total_swinging"], sw[keep]), (st["total_traction"], tr[keep])):
        want = math.fsum(vals)
        assert want > 0
        assert abs(got - want) <= 1e-12 * want, (got, want)


def test_config2_ba100k_forces(gpu, orc):
    """Config 2 at its full size: Barabasi-Albert, 100,000 nodes, m = 3,
    weights lognormal(0, 0.5), positions U[0,1000]^2, theta 1.2. Per-step
    forces from identical positions: FP64 within 1e-12 of the oracle's double
    construction; FP32 within 1e-4 of FP64 and within 1e-5 of the oracle's
    restatement of the FP32 path."""
    n, a, b = G.barabasi_albert(100_000, 3, seed=1)
    w = np.random.default_rng(1).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0.0, 1000.0, seed=3))
    go = orc.prepare_large(n, a, b, w)
    p, keep = orc.full_params(go, theta=1.2, scaling=2.0)
    want_d = orc.pipe_forces(p, pos, "d")
    with make_layout(n, a, b, w, pos, "double", theta=1.2) as L:
        fd = L.forces(pos)
    assert rel_err(fd, want_d) <= 1e-12
    with make_layout(n, a, b, w, pos, "single", theta=1.2) as L:
        ff = L.forces(pos)
        L.iterate(20)
        L.sync()
        xy = L.positions()
        ff2 = L.forces(xy)
    assert rel_err(ff, want_d) <= 1e-4
    assert rel_err(ff, orc.pipe_forces(p, pos, "m")) <= 1e-5
    # and after 20 iterations of the FP32 layout, from its own positions
    assert rel_err(ff2, orc.pipe_forces(p, xy, "d")) <= 1e-4


@pytest.mark.parametrize("opts", [dict(), dict(linlog=True), dict(adjust=True, linlog=True)])
def test_heavy_nodes_single(gpu, orc, opts):
    """FP32: nodes of 128 incidences or more (hubs) have their attraction
    summed by a warp each, in a fixed order that the oracle's restatement of
    the FP32 path mirrors: forces within 1e-5 of it, and within 1e-4 of the
    FP64 forces (2e-3 with prevent_overlap); the hub kernel is one more
    launch per iteration (and the attraction beside the walk, with its
    join, one more than the attraction fused with the totals)."""
    n, a, b = G.barabasi_albert(6000, 3, seed=12)
    rng = np.random.default_rng(13)
    hub_a = np.concatenate([np.zeros(3000, np.int32), np.ones(700, np.int32)])
    hub_b = np.concatenate([rng.choice(np.arange(2, n), 3000, replace=False),
                            rng.choice(np.arange(2, n), 700, replace=False)]).astype(np.int32)
    a, b = np.concatenate([a, hub_a]), np.concatenate([b, hub_b])
    w = rng.lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0, 1000, seed=14))
    size = f32(rng.uniform(0.5, 3.0, n)) if opts.get("adjust") else None
    go = orc.prepare_large(n, a, b, w)
    p, keep = orc.full_params(go, size=size, theta=1.2, **opts)
    with make_layout(n, a, b, w, pos, "single", size=size, theta=1.2, **opts) as L:
        f = L.forces(pos)
        heavy = L.info("heavy_nodes")
        launches = L.info("launches_per_iteration")
        L.option("overlap", 0)
        launches_fused = L.info("launches_per_iteration")
    with make_layout(n, a, b, w, pos, "double", size=size, theta=1.2, **opts) as L:
        fd = L.forces(pos)
        launches_d = L.info("launches_per_iteration")
    deg = np.diff(go.inc_off)
    assert heavy == (deg >= 128).sum() > 2
    assert launches_fused == launches_d + 1
    assert launches == launches_fused + 1
    assert rel_err(f, orc.pipe_forces(p, pos, "m")) <= 1e-5
    assert rel_err(f, fd) <= (2e-3 if opts.get("adjust") else 1e-4)


def test_fp32_forces_near_equilibrium_with_hubs(gpu):
    """Near equilibrium a hub's repulsion and attraction nearly cancel (each
    ~100 times the net force); the FP32 walk adds the terms of hubs (mass
    129 or more) with Kahan compensation, which keeps the FP32 forces within
    1e-4 of the FP64 forces at the FP32 layout's own positions after 400
    iterations (Barabasi-Albert, 20,000 nodes, lognormal weights)."""
    n, a, b = G.barabasi_albert(20000, 3, seed=21)
    w = np.random.default_rng(22).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0.0, 1000.0, seed=23))
    with make_layout(n, a, b, w, pos, "single", theta=1.2) as L:
        assert L.info("heavy_nodes") > 0
        L.iterate(400)
        L.sync()
        xy = L.positions()
        ff = L.forces(xy)
    with make_layout(n, a, b, w, xy, "double", theta=1.2) as L:
        fd = L.forces(xy)
    assert rel_err(ff, fd) <= 1e-4


@pytest.mark.parametrize("opts", [dict(), dict(linlog=True, outbound=True),
                                  dict(adjust=True, linlog=True)])
def test_attraction_beside_the_walk(gpu, orc, opts):
    """FP32 Barnes-Hut: gravity and attraction run on a second stream beside
    the tree build and the walk, into a buffer of their own, added to the
    repulsion by the join. Where the branch forks (after the sort or after
    the tree) and how many blocks it has change no bit of the trajectory;
    the force query gives the iteration's forces (the oracle's FP32 mirror
    within 1e-5; 5e-3 with prevent_overlap, whose near-contact force is
    ill-conditioned in float); the attraction fused after the walk
    (overlap 0) sums in
    another order: forces within 1e-6, positions after one iteration within
    1e-6 of the layout's extent. Hubs (the warp-summed attraction) included."""
    n, a, b = G.barabasi_albert(20000, 3, seed=31)
    rng = np.random.default_rng(32)
    a = np.concatenate([a, np.zeros(400, np.int32)])
    b = np.concatenate([b, rng.choice(np.arange(1, n), 400, replace=False).astype(np.int32)])
    w = rng.lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0, 1000, seed=33))
    adjust = opts.get("adjust", False)
    size = f32(rng.uniform(0.5, 3.0, n)) if adjust else None
    kw = {k: v for k, v in opts.items() if k != "outbound"}
    go = orc.prepare_large(n, a, b, w, outbound=opts.get("outbound", False))
    p, keep = orc.full_params(go, size=size, theta=1.2, **kw)
    runs = {}
    for name, ov, grid in (("after_sort", 1, 1), ("after_tree", 2, 1), ("grid4", 1, 4),
                           ("fused", 0, 1)):
        with make_layout(n, a, b, w, pos, "single", size=size, theta=1.2,
                         outbound=opts.get("outbound", False), **kw) as L:
            assert L.info("heavy_nodes") > 0
            L.option("overlap", ov)
            L.option("attract_grid", grid)
            f = L.forces(pos)
            L.iterate(1)
            L.sync()
            xy1 = L.positions()
            L.iterate(9)
            L.sync()
            runs[name] = (f, xy1, L.positions(), L.speed())
    base = runs["after_sort"]
    for name in ("after_tree", "grid4"):
        for k in range(3):
            np.testing.assert_array_equal(runs[name][k], base[k], err_msg=name)
        assert runs[name][3] == base[3]
    assert rel_err(base[0], orc.pipe_forces(p, pos, "m")) <= (5e-3 if adjust else 1e-5)
    fused = runs["fused"]
    assert rel_err(fused[0], base[0]) <= 1e-6
    ext = np.abs(base[1]).max()
    assert np.abs(fused[1] - base[1]).max() <= 1e-6 * ext


def test_layout_options_where_they_apply(gpu):
    """The attraction beside the walk exists in single precision with the
    Barnes-Hut repulsion only: the option is refused with a message
    elsewhere. Programmatic dependent launches (option "pdl") change no bit
    of a trajectory."""
    n, a, b = G.barabasi_albert(5000, 3, seed=51)
    w = np.ones(len(a))
    pos = f32(G.uniform_positions(n, 0, 1000, seed=52))
    with make_layout(n, a, b, w, pos, "double", theta=1.2) as L:
        with pytest.raises(RuntimeError, match="single precision|Barnes-Hut"):
            L.option("overlap", 1)
        L.option("overlap", 0)
    with make_layout(n, a, b, w, pos, "single", repulsion=REPULSION_EXACT) as L:
        with pytest.raises(RuntimeError, match="single precision|Barnes-Hut"):
            L.option("overlap", 1)
    runs = []
    for pdl in (0, 1):
        with make_layout(n, a, b, w, pos, "single", theta=1.2) as L:
            L.option("pdl", pdl)
            L.iterate(10)
            L.sync()
            runs.append(L.positions())
    np.testing.assert_array_equal(runs[0], runs[1])
