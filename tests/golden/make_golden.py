"""Generate the golden fixtures of tests/golden/ from the reference itself.

Compiles the package's own C sources and pipeline.cl from the reference
checkout (oracle/Makefile, target `ref`) and records their outputs on small
seeded cases. The reference has no stored vectors of its own: its tests
compare against an R transcription with tolerances, which R being absent
here cannot run. Re-run with:

    python tests/golden/make_golden.py

Needs the reference checkout at /root/reference (this container only).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from forceatlas2_rc_gb300 import graphs as G  # noqa: E402

# option sets of the reference's tests (test-algorithm.R:19-61,
# test-gpu.R:48-57, test-large.R:30-37)
OPTION_SETS = [
    dict(),
    dict(strong=True, gravity=0.3),
    dict(linlog=True, scaling=3.0),
    dict(outbound=True, gravity=0.0),
    dict(adjust=True),
    dict(adjust=True, linlog=True, outbound=True),
    dict(scaling=5.0, gravity=3.0, theta=0.5),
    dict(jitter_tolerance=0.2),
]


def case_graph(n=60, seed=42):
    n, a, b = G.pa_test_graph(n, seed=seed)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.2, 3.0, len(a))
    size = rng.uniform(0.5, 4.0, n)
    pos = G.uniform_positions(n, -50, 50, seed=7)
    return n, a, b, w, size, pos


def opts(d, bh=False, theta=None, threads=1):
    d = dict(d)
    sc = d.pop("scaling", 10.0)
    th = d.pop("theta", 1.2)
    th = th if theta is None else theta
    return O.Opts(scaling=sc, theta=th, barnes_hut=bh, threads=threads, **d)


def main():
    O.build(ref=True, ref_src=os.environ.get("FA2_REF", "/root/reference"))
    if O.ref_lib() is None:
        raise SystemExit("the reference could not be built (no checkout?)")
    out = {}

    # 1. per-step forces of src/forceatlas2.c
    n, a, b, w, size, pos = case_graph()
    out.update(cf_n=n, cf_from=a, cf_to=b, cf_w=w, cf_size=size, cf_pos=pos)
    for k, d in enumerate(OPTION_SETS):
        for bh, th in ((False, None), (True, 0.5), (True, 1.2)):
            o = opts(d, bh, th)
            out[f"cf_{k}_{int(bh)}_{th}"] = O.forces(n, a, b, w, pos, size, o,
                                                     which="ref")
    # coincident nodes
    pc = pos.copy()
    pc[:20] = 1.0
    out["cf_coinc_pos"] = pc
    out["cf_coinc_bh"] = O.forces(n, a, b, w, pc, size, opts({}, True, 0.0),
                                  which="ref")
    out["cf_coinc_exact"] = O.forces(n, a, b, w, pc, size, opts({}),
                                     which="ref")

    # 2. C_forceatlas2 trajectories, 10 iterations
    fixed = (np.arange(n) < 5).astype(np.int32)
    for k, d in enumerate(OPTION_SETS[:6]):
        for bh in (False, True):
            o = opts(d, bh, None, threads=2)
            out[f"cl_{k}_{int(bh)}"] = O.layout(n, a, b, w, pos, size, None,
                                                10, o, which="ref")
    out["cl_fixed"] = O.layout(n, a, b, w, pos, size, fixed, 10, opts({}),
                               which="ref")
    out["cl_fixed_mask"] = fixed
    ni, ia, ib = G.islands(5, 30, 0.3, 2, seed=1)
    ip = G.uniform_positions(ni, 0.0, 1.0, seed=1)
    out.update(isl_from=ia, isl_to=ib, isl_pos=ip)
    out["isl_layout10"] = O.layout(ni, ia, ib, np.ones(len(ia)), ip,
                                   np.ones(ni), None, 10,
                                   O.Opts(scaling=2.0, gravity=1.0),
                                   which="ref")
    out["isl_forces0"] = O.forces(ni, ia, ib, np.ones(len(ia)), ip,
                                  np.ones(ni), O.Opts(scaling=2.0),
                                  which="ref")

    # 3. the quadtree of tree_build
    m_, _ = O.mass(n, a, b)
    regs, perm, pxyz = O.ref_tree(n, pc, m_)
    out.update(qt_regions=regs, qt_perm=perm, qt_pxyz=pxyz)

    # 4. the pipeline construction, float and double
    np_ = 200
    n2, a2, b2 = G.pa_test_graph(np_, seed=5)
    p2 = G.uniform_positions(n2, -50, 50, seed=9)
    p2[:30] = p2[np.tile(np.arange(3), 10)]   # equal Morton codes
    m2, _ = O.mass(n2, a2, b2)
    out.update(pb_pos=p2, pb_mass=m2, pb_from=a2, pb_to=b2)
    line = np.stack([np.arange(64, dtype=float), np.zeros(64)], axis=1)
    two = np.array([[0.0, 0.0], [1.0, 1.0]])
    # the FP32 path builds the double construction over float-rounded
    # positions
    p32 = p2.astype(np.float32).astype(np.float64)
    out["pb32_pos"] = p32
    r = O.pipe_build(n2, p32, m2, "d", which="ref")
    for k, v in r.items():
        out[f"pb32_d_{k}"] = v
    for prec in "fd":
        r = O.pipe_build(n2, p2, m2, prec, which="ref")
        for k, v in r.items():
            out[f"pb_{prec}_{k}"] = v
        r = O.pipe_build(64, line, np.ones(64), prec, which="ref")
        for k, v in r.items():
            out[f"pl_{prec}_{k}"] = v
        r = O.pipe_build(2, two, np.ones(2), prec, which="ref")
        for k, v in r.items():
            out[f"p2_{prec}_{k}"] = v

    # 5. pipeline forces and a 5-iteration run (reference blocking and
    #    `real` totals)
    w2 = np.random.default_rng(4).uniform(0.2, 3.0, len(a2))
    s2 = np.random.default_rng(6).uniform(0.5, 4.0, n2)
    out.update(pf_w=w2, pf_size=s2)
    pipe_sets = [dict(), dict(linlog=True, adjust=True, theta=0.5),
                 dict(strong=True, theta=0.0), dict(outbound=True, gravity=0.0)]
    for k, d in enumerate(pipe_sets):
        d = dict(d)
        ob = d.pop("outbound", False)
        g = O.prepare_large(n2, a2, b2, w2, outbound=ob)
        p, keep = O.full_params(g, size=s2, **d)
        for prec in "fd":
            out[f"pf_{k}_{prec}"] = O.pipe_forces(p, p2, prec, which="ref")
    g = O.prepare_large(n2, a2, b2, w2)
    fx = (np.arange(n2) % 3 == 0).astype(np.int32)
    p, keep = O.full_params(g, size=s2, fixed=fx, iterations=5)
    out["pr_fixed"] = fx
    for prec in "fd":
        out[f"pr_{prec}"] = O.pipe_run(p, p2, prec, which="ref")

    # 6. the adaptive speed on a grid of totals
    grid = []
    for nn in (2, 150, 100000):
        for sw in (0.0, 1e-3, 1.0, 50.0, 1e4):
            for tr in (1e-3, 1.0, 30.0, 1e5):
                for jt in (0.2, 1.0):
                    for sp, ef in ((1.0, 1.0), (2000.0, 0.04), (3.0, 0.5)):
                        s_, e_ = O.update_speed(nn, sw, tr, jt, sp, ef, "ref")
                        grid.append((nn, sw, tr, jt, sp, ef, s_, e_))
    out["speed_grid"] = np.array(grid)

    np.savez_compressed(os.path.join(HERE, "fa2_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "fa2_golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
