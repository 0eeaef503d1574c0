"""Python host interface of the GB300 ForceAtlas2 engine.

It mirrors the forceatlas2r R API for the paths that run on the GPU:

* ``layout_forceatlas2_large`` -- ``layout_forceatlas2_large()``
  (reference R/large.R:80-130): the whole layout on the device, Barnes-Hut
  over a Morton/Karras tree rebuilt every iteration; goes through
  ``fa2_full_run`` of the C interface, exactly as the package's
  ``C_forceatlas2_large`` does (reference src/forceatlas2.c:835-947);
* ``layout_forceatlas2_gpu`` -- ``layout_forceatlas2_gpu()``
  (reference R/gpu.R:88-139), every step on the device: exact all-pairs
  repulsion, or Barnes-Hut over the same device-built tree;
* ``gpu_devices`` -- ``gpu_devices()`` (reference R/gpu.R:143-147).

Arguments keep the R names and meanings (argument checks of
R/forceatlas2.R:205-316); the graph is given as ``n`` and a 0-based edge
list instead of an igraph object. ``Layout`` exposes the device-resident
session (include/fa2_cuda.h) for iterating, timing and parity checks.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional

import numpy as np

from . import _lib
from ._abi import FA2_FULL_NTIMES, FULL_TIME_NAMES, DevInfo, FullParams, dptr, iptr, uptr

REPULSION_BH = 0
REPULSION_EXACT = 1

__all__ = ["gpu_devices", "layout_forceatlas2_large", "layout_forceatlas2_gpu",
           "Layout", "Graph", "prepare_graph", "REPULSION_BH",
           "REPULSION_EXACT"]


def gpu_devices() -> list:
    """The CUDA devices, with the columns of the R function: name, vendor,
    platform, version, type, memory_gb, double."""
    lib = _lib.load()
    out = []
    for i in range(lib.fa2_gpu_ndevices()):
        info = DevInfo()
        if lib.fa2_gpu_device_info(i, C.byref(info)) != 0:
            continue
        out.append(dict(name=info.name.decode(), vendor=info.vendor.decode(),
                        platform=info.platform.decode(),
                        version=info.version.decode(),
                        type="GPU" if info.is_gpu else "other",
                        memory_gb=info.memory / 1073741824.0,
                        double=bool(info.has_double)))
    return out


# ---- argument handling (reference R/forceatlas2.R:205-316, :319-450) -------

def _number(x, name, lo=-math.inf, strict=False, whole=False):
    ok = isinstance(x, (int, float, np.integer, np.floating)) and \
        not isinstance(x, bool) and math.isfinite(float(x)) and \
        (float(x) > lo if strict else float(x) >= lo) and \
        (not whole or float(x) == round(float(x)))
    if not ok:
        raise ValueError(
            f"`{name}` must be a single {'whole ' if whole else ''}number "
            f"{'greater than' if strict else 'greater than or equal to'} {lo}.")
    return float(x)


def _flag(x, name):
    if not isinstance(x, (bool, np.bool_)):
        raise ValueError(f"`{name}` must be TRUE or FALSE.")
    return bool(x)


def _edges(n, edges):
    e = np.asarray(edges if edges is not None else np.zeros((0, 2)), dtype=np.int64)
    if e.size == 0:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    if e.ndim != 2 or e.shape[1] != 2:
        raise ValueError("`edges` must be an (m, 2) array of 0-based node indices.")
    if (e < 0).any() or (e >= n).any():
        bad = int(np.flatnonzero(((e < 0) | (e >= n)).any(axis=1))[0])
        raise ValueError(f"edge {bad + 1} refers to a node that does not exist")
    if e.shape[0] > (1 << 30) - 1:
        raise ValueError("too many edges")
    return e[:, 0].astype(np.int32), e[:, 1].astype(np.int32)


def edge_weights(m, weights, edge_weight_influence=1.0, normalize_weights=False,
                 invert_weights=False):
    """Weights as the package transforms them (R/forceatlas2.R:254-264)."""
    if weights is None:
        w = np.ones(m)
    else:
        try:
            w = np.asarray(weights, dtype=np.float64).reshape(-1)
        except (TypeError, ValueError):
            raise ValueError("`weights` must be a numeric vector with one value "
                             f"per edge ({m}).") from None
        if w.size != m:
            raise ValueError(f"`weights` must have one value per edge ({m}), "
                             f"not {w.size}.")
        if (~np.isfinite(w)).any() or (w < 0).any():
            raise ValueError("`weights` must contain only finite, non-negative "
                             "values.")
    if invert_weights:
        with np.errstate(divide="ignore"):
            w = np.where(w == 0, 0.0, 1.0 / np.where(w == 0, 1.0, w))
    if normalize_weights and m > 0:
        lo, hi = w.min(), w.max()
        w = (w - lo) / (hi - lo) if lo < hi else np.ones(m)
    with np.errstate(over="ignore"):
        w = np.ones(m) if edge_weight_influence == 0 else w ** edge_weight_influence
    if (~np.isfinite(w)).any():
        raise ValueError("The edge weights are too large or too small to be used.")
    return w


class Graph:
    """Inputs of the device layout, prepared as the package's
    C_forceatlas2_large prepares them (reference src/forceatlas2.c:870-902):
    mass = 1 + degree, and a symmetric CSR whose coefficient folds in the
    weight and, with dissuade_hubs, the division by the source's mass."""

    def __init__(self, n, frm, to, w, outbound=False):
        self.n = n
        frm = np.asarray(frm, dtype=np.int64)
        to = np.asarray(to, dtype=np.int64)
        w = np.asarray(w, dtype=np.float64)
        self.mass = 1.0 + np.bincount(frm, minlength=n).astype(np.float64) + \
            np.bincount(to, minlength=n).astype(np.float64)
        # masses are integers: any summation order gives the same mean
        mean = float(self.mass.sum()) / n if n > 0 else 0.0
        coef = mean if outbound else 1.0
        keep = np.flatnonzero(frm != to)
        c = coef * w[keep] / self.mass[frm[keep]] if outbound else coef * w[keep]
        owner = np.concatenate([frm[keep], to[keep]])
        other = np.concatenate([to[keep], frm[keep]])
        eidx = np.concatenate([keep, keep])
        cc = np.concatenate([c, c])
        # by node, then edge order (each (node, edge) pair is unique: no
        # self-loop is left)
        order = np.argsort(owner * max(len(frm), 1) + eidx)
        self.inc_node = np.ascontiguousarray(other[order], dtype=np.int32)
        self.inc_coef = np.ascontiguousarray(cc[order], dtype=np.float64)
        self.inc_off = np.zeros(n + 1, np.int32)
        np.cumsum(np.bincount(owner, minlength=n), out=self.inc_off[1:])
        if self.inc_node.size == 0:
            self.inc_node = np.zeros(1, np.int32)
            self.inc_coef = np.zeros(1)


def prepare_graph(n, edges, weights=None, dissuade_hubs=False, **wkw) -> Graph:
    frm, to = _edges(n, edges)
    w = edge_weights(len(frm), weights, **wkw)
    return Graph(n, frm, to, w, outbound=dissuade_hubs)


class _EdgeOnly:
    """A graph known by its edge list only (the device prepares the rest):
    placeholder arrays for the unused CSR fields of the parameters."""

    def __init__(self, n):
        self.n = n
        self.inc_off = np.zeros(n + 1, np.int32)
        self.inc_node = np.zeros(1, np.int32)
        self.inc_coef = np.zeros(1)
        self.mass = np.ones(n)


def prepare_graph_device(n, frm, to, w, dissuade_hubs=False, device=0) -> Graph:
    """Graph with masses and incidence lists prepared on the device
    (fa2cu_graph_prep); the same arrays as Graph() builds on the host."""
    frm = np.ascontiguousarray(frm, dtype=np.int32)
    to = np.ascontiguousarray(to, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    m = len(frm)
    mass = np.zeros(n)
    off = np.zeros(n + 1, np.int32)
    node = np.zeros(max(2 * m, 1), np.int32)
    coef = np.zeros(max(2 * m, 1))
    got = _lib.load().fa2cu_graph_prep(int(device), int(n), m, iptr(frm), iptr(to),
                                       dptr(w), int(dissuade_hubs), dptr(mass),
                                       iptr(off), iptr(node), dptr(coef))
    if got < 0:
        raise RuntimeError(_lib.error())
    g = Graph.__new__(Graph)
    g.n = n
    g.mass = mass
    g.inc_off = off
    g.inc_node = node[:got].copy() if got > 0 else np.zeros(1, np.int32)
    g.inc_coef = coef[:got].copy() if got > 0 else np.zeros(1)
    return g


def _params(g: Graph, size, fixed, scaling, gravity, theta, jitter, strong,
            linlog, adjust, iterations, device, use_double, profile=False):
    n = g.n
    size = np.ascontiguousarray(size, dtype=np.float64)
    fixed = np.ascontiguousarray(fixed, dtype=np.int32)
    p = FullParams()
    p.n = n
    p.inc_off, p.inc_node = iptr(g.inc_off), iptr(g.inc_node)
    p.inc_coef, p.mass = dptr(g.inc_coef), dptr(g.mass)
    p.size, p.fixed = dptr(size), iptr(fixed)
    p.any_fixed = int(fixed.any())
    p.scaling, p.gravity, p.theta = float(scaling), float(gravity), float(theta)
    p.jitter_tolerance = float(jitter)
    p.strong, p.linlog, p.adjust = int(strong), int(linlog), int(adjust)
    p.iterations = int(iterations)
    p.device, p.use_double, p.profile = int(device), int(use_double), int(profile)
    p.source = b""
    return p, (size, fixed, g)


class Layout:
    """A layout resident on the device (include/fa2_cuda.h: fa2cu_layout_*).

    ``repulsion`` is REPULSION_BH (Barnes-Hut over the Morton/Karras tree) or
    REPULSION_EXACT (every pair). Positions cross as (n, 2) float64 arrays.
    """

    def __init__(self, g: Graph, pos, *, size=None, fixed=None, scaling=2.0,
                 gravity=1.0, theta=1.2, jitter_tolerance=1.0, strong=False,
                 linlog=False, adjust=False, precision="single", device=0,
                 repulsion=REPULSION_BH):
        self.lib = _lib.load()
        self.n = n = g.n
        size = np.ones(n) if size is None else size
        fixed = np.zeros(n, np.int32) if fixed is None else fixed
        self._p, self._keep = _params(g, size, fixed, scaling, gravity, theta,
                                      jitter_tolerance, strong, linlog, adjust,
                                      0, device, precision == "double")
        xy = _cols(pos, n)
        self.h = self.lib.fa2cu_layout_open(C.byref(self._p), dptr(xy),
                                            int(repulsion))
        if not self.h:
            raise RuntimeError(_lib.error())

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(_lib.error())

    def iterate(self, iterations: int = 1):
        self._check(self.lib.fa2cu_layout_iterate(self.h, int(iterations)))

    def sync(self):
        self._check(self.lib.fa2cu_layout_sync(self.h))

    def positions(self) -> np.ndarray:
        xy = np.zeros(2 * self.n)
        self._check(self.lib.fa2cu_layout_positions(self.h, dptr(xy)))
        return xy.reshape(2, self.n).T.copy()

    def set_positions(self, pos):
        self._check(self.lib.fa2cu_layout_set_positions(
            self.h, dptr(_cols(pos, self.n))))

    def forces(self, pos) -> np.ndarray:
        """Forces of one iteration at pos (repulsion, gravity, attraction)."""
        f = np.zeros(2 * self.n)
        self._check(self.lib.fa2cu_layout_forces(self.h, dptr(_cols(pos, self.n)),
                                                 dptr(f)))
        return f.reshape(2, self.n).T.copy()

    def speed(self):
        st = np.zeros(4)
        self._check(self.lib.fa2cu_layout_speed(self.h, dptr(st)))
        return dict(speed=st[0], efficiency=st[1], total_swinging=st[2],
                    total_traction=st[3])

    @property
    def stream(self) -> int:
        return self.lib.fa2cu_layout_stream(self.h) or 0

    def phase_times(self, iterations: int = 1) -> dict:
        ms = np.zeros(FA2_FULL_NTIMES)
        self._check(self.lib.fa2cu_layout_phase_times(self.h, int(iterations),
                                                      dptr(ms)))
        return dict(zip(FULL_TIME_NAMES, ms))

    def tree(self, pos) -> dict:
        n = self.n
        key = np.zeros(n, np.uint32)
        order = np.zeros(n, np.uint32)
        child = np.zeros(2 * (n - 1), np.int32)
        rng = np.zeros(2 * (n - 1), np.int32)
        parent = np.zeros(2 * n - 1, np.int32)
        ni = np.zeros(4 * (n - 1))
        self._check(self.lib.fa2cu_layout_tree(
            self.h, dptr(_cols(pos, n)), uptr(key), uptr(order), iptr(child),
            iptr(rng), iptr(parent), dptr(ni)))
        return dict(key=key, order=order, child=child, range=rng,
                    parent=parent, ni=ni.reshape(-1, 4))

    def traversal_counts(self):
        c = np.zeros(2)
        self._check(self.lib.fa2cu_layout_traversal_counts(self.h, dptr(c)))
        return dict(visits=c[0], pairs=c[1])

    def info(self, name: str) -> float:
        """fa2cu_layout_info: "launches_per_iteration", "heavy_nodes",
        "nodes", "incidences"."""
        v = self.lib.fa2cu_layout_info(self.h, name.encode())
        if v < 0:
            raise RuntimeError(_lib.error())
        return v

    def swing(self, traction: bool = False):
        """Per-node swinging (and traction, after option("keep_traction",
        1)) of the last iteration."""
        sw = np.zeros(self.n)
        tr = np.zeros(self.n) if traction else None
        self._check(self.lib.fa2cu_layout_swing(self.h, dptr(sw), dptr(tr)))
        return (sw, tr) if traction else sw

    def option(self, name: str, value: float):
        """Tuning option (fa2cu_layout_option), e.g. option("walk", 1)."""
        self._check(self.lib.fa2cu_layout_option(self.h, name.encode(), float(value)))

    @property
    def device_bytes(self) -> float:
        return self.lib.fa2cu_layout_bytes(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fa2cu_layout_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _cols(pos, n):
    """(n, 2) positions -> x then y (an R n x 2 matrix)."""
    pos = np.asarray(pos, dtype=np.float64)
    if pos.shape != (n, 2):
        raise ValueError(f"`init` must provide two numeric coordinates for each "
                         f"of the {n} nodes.")
    if (~np.isfinite(pos)).any():
        raise ValueError("`init` must not contain missing or infinite values.")
    return np.ascontiguousarray(pos.T.reshape(-1))


def _resolve_device(device) -> int:
    """1-based device number of the R API -> 0-based CUDA index."""
    nd = _lib.load().fa2_gpu_ndevices()
    if nd == 0:
        raise RuntimeError("No CUDA device was found: " + _lib.error())
    if device is None:
        return 0
    if isinstance(device, bool) or not isinstance(device, (int, np.integer)) or \
            device < 1 or device > nd:
        raise ValueError(f"`device` must be a device number between 1 and {nd}.")
    return int(device) - 1


def _common(n, edges, iterations, scaling_ratio, gravity, jitter_tolerance,
            theta, node_size, init, fixed, seed, weights, edge_weight_influence,
            normalize_weights, invert_weights, dissuade_hubs, flags,
            host_graph=True):
    iterations = int(_number(iterations, "iterations", 0, whole=True))
    gravity = _number(gravity, "gravity", 0)
    _number(edge_weight_influence, "edge_weight_influence", 0)
    jitter_tolerance = _number(jitter_tolerance, "jitter_tolerance", 0, strict=True)
    theta = _number(theta, "theta", 0)
    for k, v in flags.items():
        _flag(v, k)
    if scaling_ratio is None:
        scaling_ratio = 2.0 if n >= 100 else 10.0
    else:
        scaling_ratio = _number(scaling_ratio, "scaling_ratio", 0, strict=True)
    size_err = (f"`node_size` must be a single number or one finite number "
                f"per node ({n}).")
    try:
        size = np.broadcast_to(np.asarray(node_size, dtype=np.float64), (n,)).copy() \
            if np.ndim(node_size) == 0 else np.asarray(node_size, dtype=np.float64)
    except (TypeError, ValueError):
        raise ValueError(size_err) from None
    if size.shape != (n,) or (~np.isfinite(size)).any():
        raise ValueError(size_err)
    if (size < 0).any():
        raise ValueError("`node_size` must be non-negative.")
    if fixed is None:
        fx = np.zeros(n, np.int32)
    else:
        fx = np.asarray(fixed)
        if fx.shape != (n,) or fx.dtype != np.bool_:
            raise ValueError(f"`fixed` must be a logical vector with one value "
                             f"per node ({n}) and no missing value.")
        fx = fx.astype(np.int32)
    if init is None:
        if fx.any():
            raise ValueError("`fixed` nodes need a position: please provide "
                             "`init`.")
        r = 10.0 * math.sqrt(n)
        pos = np.random.default_rng(seed).uniform(-r, r, size=(n, 2))
    else:
        pos = np.asarray(init, dtype=np.float64)
        _cols(pos, n)
    frm, to = _edges(n, edges)
    w = edge_weights(len(frm), weights, edge_weight_influence=edge_weight_influence,
                     normalize_weights=normalize_weights,
                     invert_weights=invert_weights)
    # the host preparation, or the edge list for the device's
    g = Graph(n, frm, to, w, outbound=dissuade_hubs) if host_graph else \
        (frm, to, np.ascontiguousarray(w, dtype=np.float64))
    return iterations, gravity, jitter_tolerance, theta, scaling_ratio, size, \
        fx, pos, g


def layout_forceatlas2_large(n, edges, iterations=1000, scaling_ratio=None,
                             gravity=1.0, strong_gravity=False, linlog=False,
                             dissuade_hubs=False, prevent_overlap=False,
                             node_size=1.0, weights=None,
                             edge_weight_influence=1.0,
                             normalize_weights=False, invert_weights=False,
                             init=None, fixed=None, jitter_tolerance=1.0,
                             theta=1.2, device=None, precision="single",
                             seed: Optional[int] = None, timings=False,
                             prep="device"):
    """The all-GPU layout; returns an (n, 2) array (and the phase timings in
    seconds when ``timings``). ``prep="host"`` prepares masses and incidence
    lists on the host and calls ``fa2_full_run``, as the package's
    ``C_forceatlas2_large``; ``prep="device"`` (the default) passes the edge
    list to ``fa2cu_full_run_edges``, which prepares them on the device --
    the same numbers bit for bit."""
    if prep not in ("device", "host"):
        raise ValueError("`prep` must be \"device\" or \"host\"")
    if precision not in ("single", "double"):
        raise ValueError("'arg' should be one of \"single\", \"double\"")
    flags = dict(strong_gravity=strong_gravity, linlog=linlog,
                 dissuade_hubs=dissuade_hubs, prevent_overlap=prevent_overlap,
                 normalize_weights=normalize_weights,
                 invert_weights=invert_weights)
    (iterations, gravity, jitter, theta, scaling, size, fx, pos,
     g) = _common(n, edges, iterations, scaling_ratio, gravity,
                  jitter_tolerance, theta, node_size, init, fixed, seed,
                  weights, edge_weight_influence, normalize_weights,
                  invert_weights, dissuade_hubs, flags,
                  host_graph=prep == "host" or n < 2)
    if n == 0:
        return np.zeros((0, 2))
    dev = _resolve_device(device)
    if n < 2:
        # one node: the all-GPU tree needs two; the exact device layout
        # computes the same iteration
        with Layout(g, pos, size=size, fixed=fx, scaling=scaling,
                    gravity=gravity, theta=theta, jitter_tolerance=jitter,
                    strong=strong_gravity, linlog=linlog,
                    adjust=prevent_overlap, precision=precision, device=dev,
                    repulsion=REPULSION_EXACT) as L:
            L.iterate(iterations)
            L.sync()
            return L.positions()
    xy = _cols(pos, n)
    t = np.zeros(FA2_FULL_NTIMES)
    if prep == "host":
        p, keep = _params(g, size, fx, scaling, gravity, theta, jitter,
                          strong_gravity, linlog, prevent_overlap, iterations,
                          dev, precision == "double", profile=timings)
        rc = _lib.load().fa2_full_run(C.byref(p), dptr(xy), dptr(t))
    else:
        frm, to, w = g
        p, keep = _params(_EdgeOnly(n), size, fx, scaling, gravity, theta,
                          jitter, strong_gravity, linlog, prevent_overlap,
                          iterations, dev, precision == "double",
                          profile=timings)
        rc = _lib.load().fa2cu_full_run_edges(
            C.byref(p), len(frm), iptr(frm), iptr(to), dptr(w),
            int(dissuade_hubs), dptr(xy), dptr(t))
    if rc != 0:
        raise RuntimeError(_lib.error())
    out = xy.reshape(2, n).T.copy()
    if timings:
        return out, dict(zip(FULL_TIME_NAMES, t))
    return out


def layout_forceatlas2_gpu(n, edges, iterations=1000, scaling_ratio=None,
                           gravity=1.0, strong_gravity=False, linlog=False,
                           dissuade_hubs=False, prevent_overlap=False,
                           node_size=1.0, weights=None,
                           edge_weight_influence=1.0, normalize_weights=False,
                           invert_weights=False, init=None, fixed=None,
                           jitter_tolerance=1.0, barnes_hut=None, theta=1.2,
                           device=None, precision="single",
                           seed: Optional[int] = None):
    """The GPU layout: exact repulsion below 10000 nodes by default
    (reference R/forceatlas2.R:239-244), Barnes-Hut over the device tree
    above; every step of every iteration on the device."""
    if precision not in ("single", "double"):
        raise ValueError("'arg' should be one of \"single\", \"double\"")
    flags = dict(strong_gravity=strong_gravity, linlog=linlog,
                 dissuade_hubs=dissuade_hubs, prevent_overlap=prevent_overlap,
                 normalize_weights=normalize_weights,
                 invert_weights=invert_weights)
    (iterations, gravity, jitter, theta, scaling, size, fx, pos,
     g) = _common(n, edges, iterations, scaling_ratio, gravity,
                  jitter_tolerance, theta, node_size, init, fixed, seed,
                  weights, edge_weight_influence, normalize_weights,
                  invert_weights, dissuade_hubs, flags)
    if barnes_hut is None:
        barnes_hut = n >= 10000
    barnes_hut = _flag(barnes_hut, "barnes_hut")
    if n == 0:
        return np.zeros((0, 2))
    dev = _resolve_device(device)
    rep = REPULSION_BH if (barnes_hut and n >= 2) else REPULSION_EXACT
    with Layout(g, pos, size=size, fixed=fx, scaling=scaling, gravity=gravity,
                theta=theta, jitter_tolerance=jitter, strong=strong_gravity,
                linlog=linlog, adjust=prevent_overlap, precision=precision,
                device=dev, repulsion=rep) as L:
        L.iterate(iterations)
        L.sync()
        return L.positions()
