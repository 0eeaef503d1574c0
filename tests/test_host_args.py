"""Host-side argument handling of the Python mirror of the R functions, on
the CPU (no device call is reached): the checks and messages of the
reference's tests/testthat/test-interface.R:92-114, test-gpu.R:15-32 and
test-large.R:144-145, and the weight transforms of R/forceatlas2.R:254-264
(test-interface.R:80-90)."""
import numpy as np
import pytest

from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300 import layout_forceatlas2_gpu, layout_forceatlas2_large
from forceatlas2_rc_gb300 import _lib
from forceatlas2_rc_gb300.layout import edge_weights, prepare_graph

N, A, B = G.pa_test_graph(10, seed=42)
EDGES = np.column_stack([A, B])
M = len(A)

BAD = [
    (dict(iterations=-1), "iterations"),
    (dict(iterations=1.5), "iterations"),
    (dict(scaling_ratio=0), "scaling_ratio"),
    (dict(gravity=-1), "gravity"),
    (dict(gravity=float("nan")), "gravity"),
    (dict(theta=-1), "theta"),
    (dict(jitter_tolerance=0), "jitter_tolerance"),
    (dict(edge_weight_influence=-1), "edge_weight_influence"),
    (dict(linlog=None), "linlog"),
    (dict(strong_gravity="yes"), "strong_gravity"),
    (dict(prevent_overlap=1), "prevent_overlap"),
    (dict(node_size=[1.0, 2.0]), "node_size"),
    (dict(node_size=-1.0), "node_size"),
    (dict(node_size="nope"), "node_size"),
    (dict(fixed=np.array([True, False])), "fixed"),
    (dict(fixed=np.ones(N, bool)), "init"),
    (dict(init=np.zeros((N - 1, 2))), "init"),
    (dict(init=np.full((N, 2), np.nan)), "init"),
    (dict(weights="nope"), "weights"),
    (dict(weights=np.ones(M - 1)), "one value per edge"),
    (dict(weights=-np.ones(M)), "non-negative"),
    (dict(weights=np.where(np.arange(M) == 1, np.nan, 1.0)), "finite"),
    (dict(precision="half"), "arg"),
]


@pytest.mark.parametrize("fn", [layout_forceatlas2_gpu, layout_forceatlas2_large])
@pytest.mark.parametrize("kw,msg", BAD, ids=[b[1] + str(i) for i, b in enumerate(BAD)])
def test_invalid_arguments_give_clear_errors(fn, kw, msg):
    kw = dict(kw)
    with pytest.raises(ValueError, match=msg):
        fn(N, EDGES, iterations=kw.pop("iterations", 5), **kw)


def test_invalid_edges():
    with pytest.raises(ValueError, match="edge 2 refers to a node"):
        layout_forceatlas2_large(3, [[0, 1], [1, 3]], 5)
    with pytest.raises(ValueError, match="edges"):
        layout_forceatlas2_large(3, np.zeros((2, 3)), 5)
    with pytest.raises(ValueError, match="barnes_hut"):
        layout_forceatlas2_gpu(N, EDGES, 5, barnes_hut="yes")


def test_device_errors():
    """test-gpu.R:15-32: without a device the call says so; with one, a
    device number out of range is refused."""
    nd = _lib.load().fa2_gpu_ndevices()
    if nd == 0:
        with pytest.raises(RuntimeError, match="No CUDA device"):
            layout_forceatlas2_gpu(N, EDGES, 5)
        with pytest.raises(RuntimeError, match="No CUDA device"):
            layout_forceatlas2_large(N, EDGES, 5)
    else:
        for dev in (nd + 1, 0, "a"):
            with pytest.raises(ValueError, match="device"):
                layout_forceatlas2_gpu(N, EDGES, 5, device=dev)
            with pytest.raises(ValueError, match="device"):
                layout_forceatlas2_large(N, EDGES, 5, device=dev)


def test_empty_graph_needs_no_device():
    assert layout_forceatlas2_large(0, None, 5).shape == (0, 2)
    assert layout_forceatlas2_gpu(0, None, 5).shape == (0, 2)


def test_weight_transforms():
    """R/forceatlas2.R:254-264 as test-interface.R:80-90 pins them."""
    w = np.random.default_rng(1).uniform(0.5, 3.0, M)
    np.testing.assert_array_equal(edge_weights(M, None), np.ones(M))
    np.testing.assert_array_equal(edge_weights(M, w), w)
    np.testing.assert_array_equal(edge_weights(M, w, edge_weight_influence=0), np.ones(M))
    np.testing.assert_array_equal(edge_weights(M, w, invert_weights=True), 1.0 / w)
    np.testing.assert_array_equal(
        edge_weights(M, w, normalize_weights=True),
        (w - w.min()) / (w.max() - w.min()))
    np.testing.assert_array_equal(
        edge_weights(M, np.full(M, 3.0), normalize_weights=True), np.ones(M))
    w0 = w.copy()
    w0[0] = 0.0
    want = 1.0 / np.where(w0 == 0, 1.0, w0)
    want[0] = 0.0
    np.testing.assert_array_equal(edge_weights(M, w0, invert_weights=True), want)
    np.testing.assert_array_equal(edge_weights(M, w, edge_weight_influence=0.5),
                                  w ** 0.5)
    with pytest.raises(ValueError, match="too large or too small"):
        edge_weights(2, [1e300, 1.0], edge_weight_influence=2.0)


def test_host_graph_preparation():
    """Masses 1 + degree (self-loops twice), the symmetric incidence lists in
    edge order with the coefficient folding weight and (dissuade_hubs) the
    source's mass over the mean mass (reference src/forceatlas2.c:870-902)."""
    edges = np.array([[0, 1], [2, 2], [1, 2], [0, 1]])
    w = np.array([1.0, 5.0, 2.0, 4.0])
    g = prepare_graph(3, edges, w)
    np.testing.assert_array_equal(g.mass, [3.0, 4.0, 4.0])
    np.testing.assert_array_equal(g.inc_off, [0, 2, 5, 6])
    np.testing.assert_array_equal(g.inc_node, [1, 1, 0, 2, 0, 1])
    np.testing.assert_array_equal(g.inc_coef, [1.0, 4.0, 1.0, 2.0, 4.0, 2.0])
    h = prepare_graph(3, edges, w, dissuade_hubs=True)
    mean = 11.0 / 3.0
    np.testing.assert_array_equal(
        h.inc_coef, [mean * 1.0 / 3.0, mean * 4.0 / 3.0, mean * 1.0 / 3.0,
                     mean * 2.0 / 4.0, mean * 4.0 / 3.0, mean * 2.0 / 4.0])
