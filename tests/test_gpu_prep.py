"""The graph preparation on the device (fa2cu_graph_prep,
fa2cu_layout_open_edges, fa2cu_full_run_edges) against the host preparation
(Graph(), itself pinned to the reference by tests/test_prep_golden.py): bit
for bit, at sizes that need one to four 8-bit sort passes, with self-loops
and repeated edges; and whole layouts from edge lists equal to the host
path's."""
import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300.layout import (Graph, layout_forceatlas2_large,
                                         prepare_graph_device)

pytestmark = pytest.mark.gpu


def same(a, b):
    ninc = int(b.inc_off[-1])
    np.testing.assert_array_equal(a.mass, b.mass)
    np.testing.assert_array_equal(a.inc_off, b.inc_off)
    np.testing.assert_array_equal(a.inc_node[:ninc], b.inc_node[:ninc])
    np.testing.assert_array_equal(a.inc_coef[:ninc], b.inc_coef[:ninc])


@pytest.mark.parametrize("n,m", [(200, 3000), (60000, 400000), (3_000_000, 2_000_000),
                                 ((1 << 24) + 3, 1_000_000)])
def test_device_prep_equals_host(gpu, n, m):
    rng = np.random.default_rng(n)
    a = rng.integers(0, n, m).astype(np.int32)
    b = rng.integers(0, n, m).astype(np.int32)
    a[::50] = b[::50]  # self-loops
    k = m // 100       # repeated pairs, in the other direction
    a, b = np.concatenate([a, b[:k]]), np.concatenate([b, a[:k]])
    w = rng.lognormal(0.0, 0.5, len(a))
    for ob in (False, True):
        same(prepare_graph_device(n, a, b, w, dissuade_hubs=ob),
             Graph(n, a, b, w, outbound=ob))


def test_device_prep_bad_edge(gpu):
    a = np.arange(10, dtype=np.int32)
    b = a.copy()
    b[6] = 10
    b[8] = -1
    with pytest.raises(RuntimeError, match="edge 7 refers to a node that does not exist"):
        prepare_graph_device(10, a, b, np.ones(10))


@pytest.mark.parametrize("precision", ["single", "double"])
def test_full_run_edges_equals_host_path(gpu, precision):
    """layout_forceatlas2_large from the edge list (device preparation) and
    through fa2_full_run (host preparation, the package's path): the same
    positions bit for bit."""
    n, a, b = G.sbm(30000, 30, 2.1, 12.0, 2.0, seed=3)
    a = np.concatenate([a, np.arange(0, n, 1000)])   # self-loops
    b = np.concatenate([b, np.arange(0, n, 1000)])
    edges = np.stack([a, b], 1)
    w = np.random.default_rng(1).lognormal(0.0, 0.5, len(a))
    init = G.uniform_positions(n, -500, 500, seed=4)
    kw = dict(iterations=30, weights=w, dissuade_hubs=True, linlog=True,
              init=init, precision=precision)
    dev = layout_forceatlas2_large(n, edges, prep="device", **kw)
    host = layout_forceatlas2_large(n, edges, prep="host", **kw)
    np.testing.assert_array_equal(dev, host)
