"""The synthetic inputs of bench.py have the shapes of the configurations they
stand in for (no public dataset is named): the batch of config 4, the
serving trace of config 5, the Barabasi-Albert graph of config 2 and the SBM
of config 3 (at a reduced size here; the full size is built by the bench)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_batch_plan_config4():
    """4096 graphs, sizes log-uniform in [50, 20000], mean degree uniform in
    [4, 16]; Erdos-Renyi and island graphs alternately."""
    plan = bench.batch_plan(4096)
    assert len(plan) == 4096
    sizes = np.array([n for _, n, _ in plan])
    degs = np.array([d for *_, d in plan])
    assert sizes.min() >= 50 and sizes.max() <= 20000
    logs = np.log(sizes)
    # log-uniform: the logs' mean and spread of a uniform law on [ln 50, ln 20000]
    lo, hi = np.log(50.0), np.log(20000.0)
    assert abs(logs.mean() - (lo + hi) / 2) < 0.1
    assert abs(logs.std() - (hi - lo) / np.sqrt(12)) < 0.1
    assert degs.min() >= 4.0 and degs.max() <= 16.0
    assert abs(degs.mean() - 10.0) < 0.3
    graphs = bench.batch_graphs(plan[:4])
    for (i, n, deg), (g, pos) in zip(plan[:4], graphs):
        assert g.n == n and pos.shape == (n, 2)
        assert abs(2.0 * (g.mass - 1.0).sum() / 2.0 / n - deg) < 0.35 * deg + 1.0


def test_serve_trace_config5():
    """Poisson arrivals at 200/s; sizes log-uniform in [1e3, 2e6]; a 50/50
    mix of BA (m 2..5) and SBM jobs; 30 % continuations, 10 % pinned;
    iterations uniform in [200, 1000]."""
    jobs = bench.serve_trace(4000, 200.0)
    t = np.array([j["t"] for j in jobs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1.0 / 200) < 0.1 / 200
    assert abs(gaps.std() - 1.0 / 200) < 0.15 / 200  # exponential: sd = mean
    sizes = np.array([j["n"] for j in jobs])
    assert sizes.min() >= 1000 and sizes.max() <= 2_000_000
    lo, hi = np.log(1e3), np.log(2e6)
    assert abs(np.log(sizes).mean() - (lo + hi) / 2) < 0.15
    kinds = np.array([j["kind"] == "ba" for j in jobs])
    assert abs(kinds.mean() - 0.5) < 0.03
    ms = np.array([j["m"] for j in jobs])
    assert set(ms) == {2, 3, 4, 5}
    assert abs(np.mean([j["cont"] for j in jobs]) - 0.3) < 0.03
    assert abs(np.mean([j["pin"] for j in jobs]) - 0.1) < 0.02
    iters = np.array([j["iters"] for j in jobs])
    assert iters.min() >= 200 and iters.max() <= 1000
    assert abs(iters.mean() - 600) < 15


def test_ba_workload_config2():
    """Barabasi-Albert, m = 3 (about 3n edges), lognormal(0, 0.5) weights,
    positions in [0, 1000]^2 (the 20,000-node check size; the bench uses
    100,000)."""
    n, a, b, w, pos = bench.ba_workload(small=True)
    assert n == 20_000
    assert abs(len(a) - 3 * n) < 10
    assert (a != b).all()
    lw = np.log(w)
    assert abs(lw.mean()) < 0.02 and abs(lw.std() - 0.5) < 0.02
    assert pos.shape == (n, 2) and pos.min() >= 0.0 and pos.max() <= 1000.0


def test_sbm_workload_config3_shape():
    """The headline SBM at its check size: blocks of power-law sizes, mean
    within-block degree 12, between-block degree 2 (about 7 edges a node)."""
    n, a, b, pos = bench.make_workload(small=True)
    assert n == 20_000
    assert 6.0 * n < len(a) < 7.5 * n
    assert (a != b).all()
    assert pos.shape == (n, 2)
