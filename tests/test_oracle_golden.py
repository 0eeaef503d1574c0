"""The oracle against the golden fixtures recorded from the reference itself
(tests/golden/make_golden.py): bit for bit. Runs on any CPU."""
import numpy as np
import pytest

from golden.make_golden import OPTION_SETS, opts


def test_forces_match_reference_bitwise(golden, orc):
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    for k, d in enumerate(OPTION_SETS):
        for bh, th in ((False, None), (True, 0.5), (True, 1.2)):
            f = orc.forces(n, a, b, w, pos, size, opts(d, bh, th))
            np.testing.assert_array_equal(f, g[f"cf_{k}_{int(bh)}_{th}"])


def test_coincident_nodes(golden, orc):
    g = golden
    n = int(g["cf_n"])
    a, b, w, size = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"]
    pc = g["cf_coinc_pos"]
    np.testing.assert_array_equal(
        orc.forces(n, a, b, w, pc, size, opts({}, True, 0.0)), g["cf_coinc_bh"])
    np.testing.assert_array_equal(
        orc.forces(n, a, b, w, pc, size, opts({})), g["cf_coinc_exact"])
    # theta = 0 never approximates: BH == exact (test-algorithm.R:63-75)
    np.testing.assert_allclose(g["cf_coinc_bh"], g["cf_coinc_exact"],
                               rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("threads", [1, 2])
def test_layout_trajectories(golden, orc, threads):
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    for k, d in enumerate(OPTION_SETS[:6]):
        for bh in (False, True):
            got = orc.layout(n, a, b, w, pos, size, None, 10,
                             opts(d, bh, None, threads=threads))
            np.testing.assert_array_equal(got, g[f"cl_{k}_{int(bh)}"])
    got = orc.layout(n, a, b, w, pos, size, g["cl_fixed_mask"], 10, opts({}))
    np.testing.assert_array_equal(got, g["cl_fixed"])
    fixed = g["cl_fixed_mask"].astype(bool)
    np.testing.assert_array_equal(got[fixed], pos[fixed])


def test_islands(golden, orc):
    g = golden
    ia, ib, ip = g["isl_from"], g["isl_to"], g["isl_pos"]
    n = len(ip)
    o = orc.Opts(scaling=2.0, gravity=1.0)
    np.testing.assert_array_equal(
        orc.layout(n, ia, ib, np.ones(len(ia)), ip, np.ones(n), None, 10, o),
        g["isl_layout10"])
    np.testing.assert_array_equal(
        orc.forces(n, ia, ib, np.ones(len(ia)), ip, np.ones(n), o),
        g["isl_forces0"])


def test_quadtree(golden, orc):
    g = golden
    n = int(g["cf_n"])
    m, _ = orc.mass(n, g["cf_from"], g["cf_to"])
    qt = orc.QuadTree(n, g["cf_coinc_pos"], m)
    np.testing.assert_array_equal(qt.regions(), g["qt_regions"])
    np.testing.assert_array_equal(qt.perm, g["qt_perm"])
    np.testing.assert_array_equal(np.concatenate([qt.px, qt.py, qt.pm]),
                                  g["qt_pxyz"])


@pytest.mark.parametrize("prec", ["f", "d"])
def test_pipeline_construction(golden, orc, prec):
    g = golden
    cases = [("pb", g["pb_pos"], g["pb_mass"]),
             ("pl", np.stack([np.arange(64.0), np.zeros(64)], 1), np.ones(64)),
             ("p2", np.array([[0.0, 0.0], [1.0, 1.0]]), np.ones(2))]
    for tag, pos, m in cases:
        r = orc.pipe_build(len(pos), pos, m, prec)
        for k in ("key", "order", "child", "range", "parent", "ni"):
            np.testing.assert_array_equal(r[k], g[f"{tag}_{prec}_{k}"],
                                          err_msg=f"{tag} {k}")


@pytest.mark.parametrize("prec", ["f", "d"])
def test_pipeline_forces_and_run(golden, orc, prec):
    g = golden
    pos, a, b = g["pb_pos"], g["pb_from"], g["pb_to"]
    n = len(pos)
    w, s = g["pf_w"], g["pf_size"]
    sets = [dict(), dict(linlog=True, adjust=True, theta=0.5),
            dict(strong=True, theta=0.0), dict(outbound=True, gravity=0.0)]
    for k, d in enumerate(sets):
        d = dict(d)
        ob = d.pop("outbound", False)
        gr = orc.prepare_large(n, a, b, w, outbound=ob)
        p, keep = orc.full_params(gr, size=s, **d)
        np.testing.assert_array_equal(orc.pipe_forces(p, pos, prec),
                                      g[f"pf_{k}_{prec}"])
    gr = orc.prepare_large(n, a, b, w)
    p, keep = orc.full_params(gr, size=s, fixed=g["pr_fixed"], iterations=5)
    np.testing.assert_array_equal(orc.pipe_run(p, pos, prec, totals_fp64=False),
                                  g[f"pr_{prec}"])


def test_speed_update(golden, orc):
    for row in golden["speed_grid"]:
        nn, sw, tr, jt, sp, ef, s_, e_ = row
        assert orc.update_speed(int(nn), sw, tr, jt, sp, ef) == (s_, e_)
