"""The layout server (fa2cu_server_*): continuous batching of layout jobs.

Bars:
  - every job's final positions equal, bit for bit, those of the
    single-layout path (fa2cu_layout_*) for the same inputs, whether the job
    ran alone or among others of other sizes, precisions and settings;
  - the summed footprint of the resident jobs never exceeds the budget;
  - invalid jobs and jobs larger than the whole budget are refused at
    submission; a job whose numbers become invalid fails alone, with the
    reference's message, and the others complete.
"""
import threading

import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300.layout import REPULSION_BH, REPULSION_EXACT, Graph, Layout
from forceatlas2_rc_gb300.serve import Server, footprint

pytestmark = pytest.mark.gpu


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def job(kind, n, seed):
    if kind == "ba":
        n, a, b = G.barabasi_albert(n, 3, seed=seed)
    else:
        n, a, b = G.sbm(n, max(2, n // 500), 2.1, 12.0, 2.0, seed=seed)
    w = np.random.default_rng(seed).lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0.0, 1000.0, seed=seed + 1))
    return Graph(n, a, b, w), pos


def settings(k, n):
    rng = np.random.default_rng(100 + k)
    base = [dict(), dict(linlog=True, scaling=5.0), dict(strong=True, gravity=0.5),
            dict(adjust=True, size=f32(rng.uniform(1.0, 5.0, n))),
            dict(fixed=(np.arange(n) % 97 == 0).astype(np.int32))][k % 5]
    return dict(base)


def single(g, pos, iters, precision, repulsion, **kw):
    with Layout(g, pos, precision=precision, repulsion=repulsion, **kw) as L:
        L.iterate(iters)
        L.sync()
        return L.positions()


CASES = [  # kind, n, seed, iterations, precision, repulsion
    ("ba", 3000, 1, 40, "single", REPULSION_BH),
    ("sbm", 50000, 2, 25, "single", REPULSION_BH),
    ("ba", 800, 3, 60, "double", REPULSION_EXACT),
    ("ba", 20000, 4, 30, "double", REPULSION_BH),
    ("sbm", 8000, 5, 50, "single", REPULSION_BH),
    ("ba", 300, 6, 100, "single", REPULSION_EXACT),
    ("ba", 120000, 7, 20, "single", REPULSION_BH),
    ("sbm", 2500, 8, 35, "double", REPULSION_BH),
]


def test_server_results_equal_single_layout(gpu):
    """Eight jobs of 300 to 120,000 nodes (FP32 and FP64, Barnes-Hut and
    exact, linlog / strong gravity / prevent_overlap / fixed nodes) submitted
    together to a server that keeps up to 8 resident, with a chunk of 7
    iterations: each result equals the single-layout path's bit for bit; the
    same jobs one at a time (max_jobs 1) give the same results."""
    jobs = []
    for k, (kind, n, seed, it, prec, rep) in enumerate(CASES):
        g, pos = job(kind, n, seed)
        jobs.append((g, pos, it, prec, rep, settings(k, g.n)))
    want = [single(g, pos, it, prec, rep, **kw) for g, pos, it, prec, rep, kw in jobs]
    for max_jobs in (8, 1):
        with Server(max_jobs=max_jobs, chunk=7) as S:
            ids = [S.submit(g, pos, it, precision=prec, repulsion=rep, **kw)
                   for g, pos, it, prec, rep, kw in jobs]
            for k, jid in enumerate(ids):
                got, xy, info = S.wait(jid)
                assert got == jid
                np.testing.assert_array_equal(xy, want[k], err_msg=f"job {k}")
                assert info["t_submit"] <= info["t_resident"] <= info["t_end"]
            st = S.stats()
            assert st["done"] == len(jobs) and st["resident"] == 0
            assert st["footprint"] == 0


def test_server_admission_by_footprint(gpu):
    """A budget of 2.5 jobs' footprint: never more than two of six equal
    jobs are resident, and all complete."""
    g, pos = job("ba", 20000, 11)
    fp = footprint(g.n, len(g.inc_node), precision="single")
    with Server(hbm_budget=2.5 * fp, max_jobs=8, chunk=5) as S:
        ids = [S.submit(g, pos, 40) for _ in range(6)]
        res = [S.wait() for _ in ids]
        st = S.stats()
    assert sorted(r[0] for r in res) == ids
    assert st["peak_footprint"] <= 2.5 * fp
    assert st["peak_footprint"] >= 2 * fp  # two ran side by side
    first = res[0][1]
    for _, xy, _ in res[1:]:
        np.testing.assert_array_equal(xy, first)
    # a job admitted after the first two waited for one of them to end
    info = sorted((r[2] for r in res), key=lambda m: m["t_resident"])
    assert info[2]["t_resident"] >= min(info[0]["t_end"], info[1]["t_end"])


def test_server_refusals_and_failures(gpu):
    g, pos = job("ba", 5000, 12)
    fp = footprint(g.n, len(g.inc_node), precision="single")
    with Server(hbm_budget=0.5 * fp) as S:
        with pytest.raises(RuntimeError, match="budget"):
            S.submit(g, pos, 10)
    with Server() as S:
        bad = Graph(100, [0], [1], [1.0])
        bad.inc_node = np.array([500, 0], np.int32)  # a neighbour out of range
        with pytest.raises(RuntimeError, match="incidence"):
            S.submit(bad, pos[:100], 10)
        with pytest.raises(ValueError, match="infinite"):
            S.submit(g, np.full_like(pos, np.nan), 10)
        # an infinite scaling ratio makes the forces invalid: that job fails,
        # the others complete
        _, sa, sb = G.erdos_renyi(50, 4.0, seed=3)
        small = Graph(50, sa, sb, np.ones(len(sa)))
        ok1 = S.submit(g, pos, 20)
        badj = S.submit(small, pos[:50], 20, scaling=np.inf, repulsion=REPULSION_EXACT)
        ok2 = S.submit(g, pos, 20)
        with pytest.raises(RuntimeError, match="invalid numbers"):
            S.wait(badj)
        a = S.wait(ok1)
        b = S.wait(ok2)
        np.testing.assert_array_equal(a[1], b[1])
        with pytest.raises(RuntimeError, match="no job"):
            S.wait(timeout=0.01)
        st = S.stats()
        assert st["failed"] == 1 and st["done"] == 2


def test_server_threads_submit_concurrently(gpu):
    """Four host threads submit and collect their own jobs at once."""
    g, pos = job("ba", 4000, 21)
    want = single(g, pos, 30, "single", REPULSION_BH)
    errors = []
    with Server(max_jobs=4, chunk=4) as S:
        def worker():
            try:
                ids = [S.submit(g, pos, 30) for _ in range(3)]
                for jid in ids:
                    _, xy, _ = S.wait(jid)
                    np.testing.assert_array_equal(xy, want)
            except Exception as e:  # reported below
                errors.append(e)
        ts = [threading.Thread(target=worker) for _ in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        assert S.stats()["done"] == 12
    assert not errors, errors


def test_footprint_matches_allocation(gpu):
    """The admission estimate equals the bytes a layout allocates plus the
    staging of its graph upload."""
    for prec in ("single", "double"):
        for rep in (REPULSION_BH, REPULSION_EXACT):
            for adjust in (False, True):
                g, pos = job("ba", 3000, 31)
                with Layout(g, pos, precision=prec, repulsion=rep, adjust=adjust) as L:
                    held = L.device_bytes
                ninc = int(g.inc_off[-1])
                staging = max(g.n, ninc) * 8 + ninc * 4
                assert footprint(g.n, ninc, adjust, False, prec, rep) == held + staging


def test_server_least_work_first(gpu):
    """With one resident job at a time and the least-work policy, jobs queued
    behind a running one are admitted smallest first; results are unchanged."""
    big, bpos = job("sbm", 60000, 41)
    small = [job("ba", 2000, 42 + k) for k in range(3)]
    want_big = single(big, bpos, 40, "single", REPULSION_BH)
    with Server(max_jobs=1, chunk=4, policy="least_work") as S:
        blocker = S.submit(big, bpos, 200)  # resident while the others queue
        ids = [S.submit(big, bpos, 40)] + [S.submit(g, p, 40) for g, p in small]
        S.wait(blocker)
        res = {jid: S.wait(jid) for jid in ids}
    order = sorted(ids, key=lambda j: res[j][2]["t_resident"])
    assert order[-1] == ids[0], order  # the big job last
    np.testing.assert_array_equal(res[ids[0]][1], want_big)
    with pytest.raises(ValueError):
        Server(policy="random")


def test_served_jobs_match_oracle(gpu, orc):
    """One served FP64 job of each kind, submitted together, against the
    oracle's restatement of the all-GPU pipeline (pipeline.cl in double,
    FP64 totals) rather than another CUDA path: a Barabasi-Albert job, an SBM
    job with linlog, a continuation from stored coordinates with
    prevent_overlap and node sizes U[1,5], and a job that pins its top-1%
    degree nodes. Positions after 12 iterations within 1e-9."""
    specs = [("ba", 1800, 61, {}), ("sbm", 2000, 62, dict(linlog=True)),
             ("ba", 1500, 63, "continuation"), ("sbm", 5000, 64, "pinned")]
    jobs = []
    for kind, n, seed, extra in specs:
        if kind == "ba":
            n, a, b = G.barabasi_albert(n, 3, seed=seed)
        else:
            n, a, b = G.sbm(n, max(2, n // 500), 2.1, 12.0, 2.0, seed=seed)
        w = np.random.default_rng(seed).lognormal(0.0, 0.5, len(a))
        g = Graph(n, a, b, w)
        pos = f32(G.uniform_positions(n, 0.0, 1000.0, seed=seed + 1))
        kw = dict(scaling=2.0, gravity=1.0, theta=1.2)
        if extra == "continuation":
            pos = single(g, pos, 30, "double", REPULSION_BH, **kw)  # stored coordinates
            kw.update(adjust=True, size=f32(np.random.default_rng(seed).uniform(1, 5, n)))
        elif extra == "pinned":
            top = np.argsort(-(g.mass - 1.0), kind="stable")[:max(1, n // 100)]
            fixed = np.zeros(n, np.int32)
            fixed[top] = 1
            kw["fixed"] = fixed
        else:
            kw.update(extra)
        jobs.append((n, a, b, w, g, pos, kw))
    iters = 12
    with Server(max_jobs=4, chunk=5) as S:
        ids = [S.submit(g, pos, iters, precision="double", **kw)
               for n, a, b, w, g, pos, kw in jobs]
        got = [S.wait(jid)[1] for jid in ids]
    for k, (n, a, b, w, g, pos, kw) in enumerate(jobs):
        go = orc.prepare_large(n, a, b, w)
        p, keep = orc.full_params(go, iterations=iters, **kw)
        want = orc.pipe_run(p, pos, "d")
        np.testing.assert_allclose(got[k], want, rtol=1e-9,
                                   atol=1e-9 * np.abs(want).max(), err_msg=f"job {k}")
        if "fixed" in kw:
            np.testing.assert_array_equal(got[k][kw["fixed"] == 1], pos[kw["fixed"] == 1])
