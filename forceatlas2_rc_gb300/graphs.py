"""Seeded synthetic graphs of the shapes the layout engine is measured on.

No dataset is bundled with the package; these generators stand in for the
graph families of its benchmark configurations. Every generator returns
``(n, from_, to_)`` with 0-based ``int32`` endpoint arrays (an undirected edge
list, each edge once) and is reproducible from ``seed`` (numpy PCG64).

* ``islands``          -- k islands of s nodes, each within-island pair an
                          edge with probability p, plus a few random edges
                          between every pair of islands (the package README's
                          example graph).
* ``barabasi_albert``  -- preferential attachment, m edges per new node.
* ``sbm``              -- stochastic block model with power-law block sizes.
* ``erdos_renyi``      -- G(n, M) with a given mean degree.
* ``pa_test_graph``    -- preferential attachment with m = 2, the shape of the
                          package's own test graphs (``igraph::sample_pa``).
"""
from __future__ import annotations

import numpy as np

__all__ = ["islands", "barabasi_albert", "sbm", "erdos_renyi",
           "pa_test_graph", "uniform_positions", "dedupe"]


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def dedupe(n: int, a: np.ndarray, b: np.ndarray):
    """Drop self-loops and repeated undirected pairs; keep first occurrence
    order by sorted pair key (deterministic)."""
    a = np.asarray(a, dtype=np.int64)
    b = np.asarray(b, dtype=np.int64)
    keep = a != b
    a, b = a[keep], b[keep]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo * n + hi
    _, first = np.unique(key, return_index=True)
    first.sort()
    return a[first].astype(np.int32), b[first].astype(np.int32)


def islands(n_islands: int = 5, size: int = 30, p: float = 0.3,
            between: int = 2, seed: int = 1):
    rng = _rng(seed)
    n = n_islands * size
    iu, ju = np.triu_indices(size, k=1)
    fa, ta = [], []
    for k in range(n_islands):
        pick = rng.random(iu.size) < p
        fa.append(iu[pick] + k * size)
        ta.append(ju[pick] + k * size)
    for k in range(n_islands):
        for l in range(k + 1, n_islands):
            fa.append(rng.integers(0, size, between) + k * size)
            ta.append(rng.integers(0, size, between) + l * size)
    a, b = dedupe(n, np.concatenate(fa), np.concatenate(ta))
    return n, a, b


def barabasi_albert(n: int, m: int = 3, seed: int = 1):
    """Preferential attachment: node v >= m links to m distinct earlier nodes
    drawn with probability proportional to degree (the endpoint-list method);
    the first m nodes form a star on node m."""
    rng = _rng(seed)
    if n <= m:
        raise ValueError("barabasi_albert needs n > m")
    src = np.empty((n - m) * m, dtype=np.int32)
    dst = np.empty((n - m) * m, dtype=np.int32)
    ends = np.empty(2 * (n - m) * m + m, dtype=np.int64)
    nends = 0
    targets = list(range(m))
    u = rng.random(2 * (n - m) * m + 64)
    ui = 0
    e = 0
    for v in range(m, n):
        for t in targets:
            src[e] = v
            dst[e] = t
            e += 1
            ends[nends] = v
            ends[nends + 1] = t
            nends += 2
        chosen = set()
        while len(chosen) < m:
            if ui >= u.size:
                u = rng.random(u.size)
                ui = 0
            chosen.add(int(ends[int(u[ui] * nends)]))
            ui += 1
        targets = list(chosen)
    return n, src, dst


def barabasi_albert_fast(n: int, m: int = 3, seed: int = 1):
    """Preferential attachment for large n, vectorised: nodes join in
    batches of about 1/16 of the nodes present, each drawing m endpoints
    uniformly from the endpoint list as it stood when its batch began (the
    degree-proportional choice of barabasi_albert, up to that lag); repeated
    picks are dropped. Node m starts as the hub of a star on 0..m-1."""
    rng = _rng(seed)
    if n <= m:
        raise ValueError("barabasi_albert_fast needs n > m")
    ends = np.empty(2 * m * (n - m), dtype=np.int64)
    ends[:m] = m
    ends[m:2 * m] = np.arange(m)
    ne = 2 * m
    src = [np.full(m, m, np.int64)]
    dst = [np.arange(m, dtype=np.int64)]
    v = m + 1
    while v < n:
        b = min(n - v, max(1, v // 16))
        new = np.repeat(np.arange(v, v + b, dtype=np.int64), m)
        tgt = ends[rng.integers(0, ne, b * m)]
        src.append(new)
        dst.append(tgt)
        ends[ne:ne + b * m] = new
        ends[ne + b * m:ne + 2 * b * m] = tgt
        ne += 2 * b * m
        v += b
    a, t = dedupe(n, np.concatenate(src), np.concatenate(dst))
    return n, a, t


def pa_test_graph(n: int, seed: int = 42):
    """The package tests' graph shape: preferential attachment with m = 2."""
    if n < 3:
        return n, np.zeros(0, np.int32), np.zeros(0, np.int32)
    return barabasi_albert(n, 2, seed)


def sbm(n: int = 1_000_000, blocks: int = 1000, exponent: float = 2.1,
        deg_in: float = 12.0, deg_out: float = 2.0, seed: int = 1):
    """Block sizes from a discrete power law P(s) ~ s^-exponent rescaled to
    sum to n; deg_in/2 * s random pairs inside each block (capped at
    s(s-1)/2) and deg_out/2 * n random pairs between blocks."""
    rng = _rng(seed)
    raw = rng.zipf(exponent, blocks).astype(np.float64)
    raw = np.minimum(raw, 1e9)
    sizes = np.maximum(1, np.floor(raw / raw.sum() * n)).astype(np.int64)
    sizes[np.argmax(sizes)] += n - int(sizes.sum())
    if sizes.min() < 1:
        raise ValueError("sbm: block sizes do not fit n")
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    want = np.minimum((deg_in / 2.0 * sizes).astype(np.int64),
                      sizes * (sizes - 1) // 2)
    blk = np.repeat(np.arange(blocks), want)
    s = sizes[blk]
    a = starts[blk] + (rng.random(blk.size) * s).astype(np.int64)
    b = starts[blk] + (rng.random(blk.size) * s).astype(np.int64)
    m_out = int(deg_out / 2.0 * n)
    block_of = np.repeat(np.arange(blocks), sizes)
    ca = rng.integers(0, n, m_out)
    cb = rng.integers(0, n, m_out)
    cross = block_of[ca] != block_of[cb]
    fa, ta = dedupe(n, np.concatenate([a, ca[cross]]),
                    np.concatenate([b, cb[cross]]))
    return n, fa, ta


def erdos_renyi(n: int, mean_degree: float, seed: int = 1):
    rng = _rng(seed)
    m = int(round(mean_degree * n / 2.0))
    a = rng.integers(0, n, m)
    b = rng.integers(0, n, m)
    fa, ta = dedupe(n, a, b)
    return n, fa, ta


def island_graph(n: int, mean_degree: float, island: int = 40, seed: int = 1):
    """n nodes in islands of `island` nodes (the last one smaller); each
    within-island pair is an edge with p = mean_degree / (island - 1) (at most
    1), and every island sends 2 edges to random other islands."""
    rng = _rng(seed)
    k = max(1, -(-n // island))
    sizes = np.full(k, island, dtype=np.int64)
    sizes[-1] = n - island * (k - 1)
    iu, ju = np.triu_indices(island, k=1)
    # one draw per pair slot of every island; the last island keeps only the
    # pairs of its own nodes
    pick = rng.random((k, iu.size)) < min(1.0, mean_degree / (island - 1))
    pick &= ju[None, :] < sizes[:, None]
    c, q = np.nonzero(pick)
    fa = [iu[q] + c * island]
    ta = [ju[q] + c * island]
    if k > 1:
        src = np.repeat(np.arange(k), 2)
        dst = (src + rng.integers(1, k, src.size)) % k
        fa.append(src * island + rng.integers(0, island, src.size) % sizes[src])
        ta.append(dst * island + rng.integers(0, island, src.size) % sizes[dst])
    a, b = dedupe(n, np.concatenate(fa), np.concatenate(ta))
    return n, a, b


def uniform_positions(n: int, lo: float, hi: float, seed: int = 7):
    """Start positions uniform in [lo, hi]^2, as an (n, 2) float64 array."""
    rng = _rng(seed)
    return rng.uniform(lo, hi, size=(n, 2))
