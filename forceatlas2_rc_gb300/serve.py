"""The layout server (include/fa2_cuda.h: fa2cu_server_*).

Jobs -- one layout each, with the arguments of ``Layout`` and a number of
iterations -- are submitted from any thread and run concurrently on one GPU:
the server admits them while their estimated device footprint fits its HBM
budget, keeps each one's positions, tree and speed state resident, and
interleaves their iterations on streams of their own (continuous batching).
A job's result is the same as the single-layout path's, alone or in the mix.
The reference has no counterpart (one layout per call, start to end).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._abi import ServerConfig, dptr
from .layout import REPULSION_BH, Graph, _cols, _params


def footprint(n: int, ninc: int, adjust: bool = False, any_fixed: bool = False,
              precision: str = "single", repulsion: int = REPULSION_BH) -> float:
    """Device bytes of one resident layout (the admission estimate)."""
    return _lib.load().fa2cu_layout_footprint(int(n), int(ninc), int(adjust),
                                              int(any_fixed),
                                              int(precision == "double"),
                                              int(repulsion))


class Server:
    """A layout server on one device.

    ``hbm_budget`` (bytes; None: 80 % of the free memory) bounds the summed
    footprint of the resident jobs, ``max_jobs`` their number; ``chunk`` is
    the number of iterations enqueued per job at a time; ``policy`` the
    admission order, "arrival" or "least_work" (nodes x iterations).
    """

    POLICIES = {"arrival": 0, "least_work": 1}

    def __init__(self, device: int = 0, hbm_budget: float | None = None,
                 max_jobs: int = 16, chunk: int = 16, policy: str = "arrival"):
        self.lib = _lib.load()
        if policy not in self.POLICIES:
            raise ValueError(f"policy must be one of {sorted(self.POLICIES)}")
        cfg = ServerConfig(int(device), float(hbm_budget or 0.0), int(max_jobs),
                           int(chunk), self.POLICIES[policy])
        self.device = int(device)
        self.h = self.lib.fa2cu_server_open(C.byref(cfg))
        if not self.h:
            raise RuntimeError(_lib.error())

    def submit(self, g: Graph, pos, iterations: int, *, size=None, fixed=None,
               scaling=2.0, gravity=1.0, theta=1.2, jitter_tolerance=1.0,
               strong=False, linlog=False, adjust=False, precision="single",
               repulsion=REPULSION_BH) -> int:
        """Queue a layout job; returns its id. The arrays are copied."""
        n = g.n
        size = np.ones(n) if size is None else size
        fixed = np.zeros(n, np.int32) if fixed is None else fixed
        p, keep = _params(g, size, fixed, scaling, gravity, theta,
                          jitter_tolerance, strong, linlog, adjust, iterations,
                          self.device, precision == "double")
        xy = _cols(pos, n)
        jid = self.lib.fa2cu_server_submit(self.h, C.byref(p), dptr(xy),
                                           int(repulsion))
        if jid < 0:
            raise RuntimeError(_lib.error())
        return jid

    def wait(self, job: int | None = None, timeout: float | None = None):
        """Collect job `job` (any ended job if None) once it has ended:
        returns (id, positions (n, 2), info), or None on timeout. info holds
        the submit, resident and end times (seconds, one clock), n,
        iterations, footprint and final speed; a failed job raises
        RuntimeError with its message."""
        info = np.zeros(8)
        got = self.lib.fa2cu_server_wait(self.h, -1 if job is None else int(job),
                                         -1.0 if timeout is None else float(timeout),
                                         dptr(info))
        if got == -1:
            return None
        if got < 0:
            raise RuntimeError(_lib.error())
        n = int(info[4])
        buf = np.zeros(2 * n)
        if self.lib.fa2cu_server_collect(self.h, got, dptr(buf)) != 0:
            raise RuntimeError(f"job {got}: " + _lib.error())
        meta = dict(t_submit=info[0], t_resident=info[1], t_end=info[2],
                    n=n, iterations=int(info[5]), footprint=info[6],
                    speed=info[7], latency=info[2] - info[0],
                    queued=info[1] - info[0])
        return got, buf.reshape(2, n).T.copy(), meta

    def stats(self) -> dict:
        s = np.zeros(8)
        self.lib.fa2cu_server_stats(self.h, dptr(s))
        return dict(queued=int(s[0]), resident=int(s[1]), done=int(s[2]),
                    failed=int(s[3]), footprint=s[4], peak_footprint=s[5],
                    budget=s[6], pool_reserved=s[7])

    def close(self):
        if getattr(self, "h", None):
            self.lib.fa2cu_server_close(self.h)
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
