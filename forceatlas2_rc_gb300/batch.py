"""Many independent layouts in one launch (include/fa2_cuda.h: fa2cu_batch_*).

The reference lays out one graph per call (``C_forceatlas2`` on the CPU,
``C_forceatlas2_large`` on the GPU, src/forceatlas2.c). A collection of many
small and medium graphs -- one layout per connected component, per sample, per
request -- would then cost one call each and leave most of the GPU idle. A
``Batch`` holds all of them on the device; one persistent launch lays every
graph out with one thread block, largest first, each graph with its own
settings and its own speed state. A graph's result does not depend on the
other graphs of the batch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._abi import FullParams, dptr
from ._lib import P_D
from .layout import Graph, _cols, _params


def tune(device: int = 0, precision: str = "single") -> dict:
    """The autotuner's choice on this device: ``exact_below`` (graphs with
    fewer nodes use the all-pairs repulsion), ``threads`` per block and
    ``nodes_per_thread`` of the all-pairs sum (its tile shape). Measured once
    per device and precision, then cached."""
    lib = _lib.load()
    eb, th, npt = C.c_int(0), C.c_int(0), C.c_int(0)
    if lib.fa2cu_batch_tune(int(device), int(precision == "double"),
                            C.byref(eb), C.byref(th), C.byref(npt)) != 0:
        raise RuntimeError(_lib.error())
    return dict(exact_below=eb.value, threads=th.value, nodes_per_thread=npt.value)


class Batch:
    """Graphs laid out together on one device.

    ``graphs`` is a list of ``Graph`` (``prepare_graph``), ``pos`` a list of
    (n, 2) start positions. ``settings`` gives the keyword arguments of
    ``Layout`` (scaling, gravity, theta, jitter_tolerance, strong, linlog,
    adjust, size, fixed) for every graph; ``per_graph`` (a list of dicts, one
    per graph) overrides them graph by graph. ``exact_below`` / ``threads``
    / ``nodes_per_thread`` default to the autotuner's values.
    """

    _KEYS = ("size", "fixed", "scaling", "gravity", "theta", "jitter_tolerance",
             "strong", "linlog", "adjust")

    def __init__(self, graphs: list, pos: list, *, precision: str = "single",
                 device: int = 0, exact_below: int | None = None,
                 threads: int | None = None, nodes_per_thread: int | None = None,
                 per_graph: list | None = None,
                 **settings):
        bad = set(settings) - set(self._KEYS)
        if bad:
            raise TypeError(f"unknown setting(s): {sorted(bad)}")
        if len(graphs) != len(pos) or not graphs:
            raise ValueError("one start layout per graph, and at least one graph")
        if per_graph is not None and len(per_graph) != len(graphs):
            raise ValueError("per_graph needs one dict per graph")
        self.lib = _lib.load()
        self.sizes = [g.n for g in graphs]
        count = len(graphs)
        arr = (FullParams * count)()
        self._keep, xy = [], []
        for k, g in enumerate(graphs):
            if not isinstance(g, Graph):
                raise TypeError("graphs must be prepare_graph() results")
            o = dict(scaling=2.0, gravity=1.0, theta=1.2, jitter_tolerance=1.0,
                     strong=False, linlog=False, adjust=False, size=None,
                     fixed=None)
            o.update(settings)
            if per_graph is not None:
                o.update(per_graph[k])
            n = g.n
            size = np.ones(n) if o["size"] is None else o["size"]
            fixed = np.zeros(n, np.int32) if o["fixed"] is None else o["fixed"]
            p, keep = _params(g, size, fixed, o["scaling"], o["gravity"],
                              o["theta"], o["jitter_tolerance"], o["strong"],
                              o["linlog"], o["adjust"], 0, device,
                              precision == "double")
            arr[k] = p
            self._keep.append(keep)
            xy.append(_cols(pos[k], n))
        self._xy = xy
        ptrs = (P_D * count)(*[dptr(a) for a in xy])
        self.h = self.lib.fa2cu_batch_open(
            arr, count, ptrs, -1 if exact_below is None else int(exact_below),
            0 if threads is None else int(threads),
            0 if nodes_per_thread is None else int(nodes_per_thread))
        if not self.h:
            raise RuntimeError(_lib.error())

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(_lib.error())

    def __len__(self):
        return len(self.sizes)

    def iterate(self, iterations: int = 1):
        """Enqueue `iterations` iterations of every graph (one launch)."""
        self._check(self.lib.fa2cu_batch_iterate(self.h, int(iterations)))

    def sync(self):
        self._check(self.lib.fa2cu_batch_sync(self.h))

    def positions(self, g: int) -> np.ndarray:
        n = self.sizes[g]
        xy = np.zeros(2 * n)
        self._check(self.lib.fa2cu_batch_positions(self.h, int(g), dptr(xy)))
        return xy.reshape(2, n).T.copy()

    def forces(self, g: int) -> np.ndarray:
        """Graph g's forces of the last iteration, at the positions before
        its displacement, as an (n, 2) array (after ``sync``)."""
        n = self.sizes[g]
        f = np.zeros(2 * n)
        self._check(self.lib.fa2cu_batch_forces(self.h, int(g), dptr(f)))
        return f.reshape(2, n).T.copy()

    def speed(self, g: int) -> dict:
        st = np.zeros(4)
        self._check(self.lib.fa2cu_batch_speed(self.h, int(g), dptr(st)))
        return dict(speed=st[0], efficiency=st[1], total_swinging=st[2],
                    total_traction=st[3])

    PHASES = ("codes", "sort", "tree", "sums", "repulsion", "attraction",
              "totals", "move")

    def phase_cycles(self, iterations: int = 1) -> dict:
        """SM cycles per phase, summed over the blocks, of `iterations`
        instrumented iterations (the positions advance)."""
        c = np.zeros(8)
        self._check(self.lib.fa2cu_batch_phase_cycles(self.h, int(iterations), dptr(c)))
        return dict(zip(self.PHASES, c))

    @property
    def stream(self) -> int:
        return self.lib.fa2cu_batch_stream(self.h) or 0

    @property
    def device_bytes(self) -> float:
        return self.lib.fa2cu_batch_bytes(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fa2cu_batch_close(self.h)
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
