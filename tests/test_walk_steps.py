"""The Barnes-Hut walk's step bound on a tree built to make it long.

The per-thread walk takes one loop step per region it visits, one per single
node it reaches as a leaf of the tree, and one per node pair it sums: at most
(n - 1) + n + n steps. Its safety cap must sit above that bound, else a legal
tree ends the walk early with a bounds error.

The layout below makes nearly every walk take close to the bound at
theta = 0: 600 clusters, each of 8 coincident nodes at a multiple of 1024 on
a 64 x 64 grid plus 10 nodes offset diagonally by 1024 / 2^k (k = 1..10),
and the corners (0, 0) and (65535, 65535), so the Morton scale is exactly 1.
Each cluster's keys share long prefixes: the Karras tree hangs one single
node off every level of a deep chain, and every one of those leaves costs
two steps.
"""
import numpy as np
import pytest

from conftest import rel_err
from forceatlas2_rc_gb300.layout import Graph, Layout


def nested_chains(seed=0, clusters=600):
    rng = np.random.default_rng(seed)
    cells = rng.choice(64 * 64, clusters, replace=False)
    base = np.stack([cells % 64, cells // 64], 1).astype(float) * 1024.0
    off = 1024.0 * 2.0 ** -np.arange(1, 11)
    pts = [np.array([[0.0, 0.0], [65535.0, 65535.0]])]
    for c in base:
        pts.append(np.repeat(c[None], 8, 0))
        pts.append(c[None] + np.stack([off, off], 1))
    return np.concatenate(pts)


def walk_steps_theta0(tree, n):
    """Loop steps of the per-thread walk at theta = 0 (every region of more
    than 8 nodes is opened; smaller ones are summed node by node), counted on
    the Karras tree of the oracle. At theta = 0 every node's walk takes the
    same path."""
    nl = n - 1
    child = tree["child"].reshape(-1, 2)
    rng = tree["range"].reshape(-1, 2)
    rope = -np.ones(n, np.int64)  # position after sorted node p in preorder
    for r in range(nl):
        b = child[r, 1]
        first = b - nl if b >= nl else rng[b, 0]
        rope[first - 1] = b
    cur, steps = 0, 0
    while cur != -1:
        if cur >= nl:  # a single node: the visit, then its pair
            steps += 2
            cur = rope[cur - nl]
            continue
        steps += 1
        first, last = rng[cur]
        if last - first >= 8:
            cur = child[cur, 0]
        else:
            steps += last - first + 1
            cur = rope[last]
    return steps


def test_nested_chains_need_more_than_two_steps_per_node(orc):
    """The case is adversarial: its walks need more than 2n + 64 steps
    (the cap that used to raise a false bounds error), and stay within the
    3n bound."""
    pos = nested_chains()
    n = len(pos)
    tree = orc.pipe_build(n, pos, np.ones(n), "d")
    s = walk_steps_theta0(tree, n)
    assert 2 * n + 64 < s <= 3 * n - 1, (n, s)


def _graph(n):
    a = np.arange(n - 1, dtype=np.int32)
    return a, a + 1, np.ones(n - 1)


@pytest.mark.gpu
@pytest.mark.parametrize("theta", [0.0, 0.1])
def test_long_walks_match_oracle(gpu, orc, theta):
    """Forces on the nested-chain layout at theta 0 and 0.1: FP64 within
    1e-12 of the oracle's double construction and FP32 within 1e-5 of the
    oracle's restatement of the FP32 path, with no bounds error; a few
    iterations of the layout complete."""
    pos = nested_chains()
    n = len(pos)
    a, b, w = _graph(n)
    go = orc.prepare_large(n, a, b, w)
    p, keep = orc.full_params(go, theta=theta, scaling=2.0)
    g = Graph(n, a, b, w)
    with Layout(g, pos, precision="double", theta=theta) as L:
        fd = L.forces(pos)
        L.iterate(3)
        L.sync()
    assert rel_err(fd, orc.pipe_forces(p, pos, "d")) <= 1e-12
    with Layout(g, pos, precision="single", theta=theta) as L:
        ff = L.forces(pos)
        L.iterate(3)
        L.sync()
    assert rel_err(ff, orc.pipe_forces(p, pos, "m")) <= 1e-5
