#!/usr/bin/env python
"""Throughput of the ForceAtlas2 iteration on GB300 (node-iterations/s).

Headline workload (the line's value): stochastic block model, 1,000,000
nodes in 1,000 blocks of power-law sizes (exponent 2.1), mean within-block
degree 12, mean between-block degree 2 (~7M edges), unit weights; linlog +
dissuade_hubs, Barnes-Hut theta 1.2, positions and forces in FP32,
swing/traction totals and the speed controller in FP64. Synthetic, generated
from a seed.

One step = one ForceAtlas2 iteration of the whole graph (Morton codes, radix
sort, Karras tree, Barnes-Hut repulsion, attraction and gravity, swing and
traction, displacement), with the graph already resident in HBM. The
iteration's working set (~0.3 GB) exceeds the 129 MB L2, so no flush is
needed between steps.

Beside the headline, the same line carries the other configurations as
objects of their own: "ba100k" (Barabasi-Albert, 100,000 nodes, 500
iterations, FP32 against FP64), "batch" (4096 graphs in one persistent
launch against one graph at a time), "serve" (the layout server on a
Poisson trace at 200 requests/s and at 0.8 x its capacity: p50/p99) and
"gpu_mode" (the reference's `_gpu` mode: CPU quadtree per iteration plus
this library's repulsion backend). --no-extras leaves them out.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sbm1m|ba100k|exact|batch|serve]

--impl reference times the reference's CPU engine (src/forceatlas2.c's
C_forceatlas2 loop with the Gephi quadtree, OpenMP on every host core; the
oracle's restatement, since the reference sources are not on the GPU host)
on the same workload. With N > 1 (torchrun), each rank lays out its own
replica on its own GPU (the layouts are independent: no collective on the
data path); value is the sum over ranks, timed by the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("node-iters/s FP32 vs FP64 at ≤1e-4 force err; served layouts/s, "
          "p99 latency")
UNIT = "node-iters/s"
WORKLOAD = ("SBM n=1,000,000, 1000 power-law blocks (exp 2.1), deg_in 12, "
            "deg_out 2, unit weights; linlog + dissuade_hubs, Barnes-Hut "
            "theta 1.2, FP32 positions/forces, FP64 speed control")
# Barnes-Hut walks (fa2cu_layout_option "walk"): the same regions and node
# pairs (the deferred walk adds them up in another order)
WALKS = {"warp": 0, "thread": 1, "wide": 2, "pair": 3, "quad": 4, "deferred": 5}
# algorithmic HBM bytes per node of the traversal: psort record 16, order 4,
# force write 8 (FP32)
TRAVERSE_HBM_BYTES_PER_NODE = 28
# L2 request bytes of the walk: a region's two records (16 + 8 bytes), a
# node pair's psort record (16 bytes)
TRAVERSE_L2_BYTES_PER_VISIT = 24
TRAVERSE_L2_BYTES_PER_PAIR = 16
# DRAM bytes (read + write) of one traversal launch on this workload
# (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture of each
# walk), and the share of cycles the schedulers issued (the kernel's bound)
TRAVERSE_DRAM_BYTES = {"deferred": 53.06e6 + 4.54e6, "thread": 45.94e6 + 0.86e6}
TRAVERSE_ISSUE_ACTIVE = {"deferred": 0.757, "thread": 0.805}
# and its L1 throughput (share of peak, same captures)
TRAVERSE_L1_THROUGHPUT = {"deferred": 0.859, "thread": 0.78}


def make_workload(small: bool = False):
    from forceatlas2_rc_gb300 import graphs
    if small:
        n, a, b = graphs.sbm(20000, 50, 2.1, 12.0, 2.0, seed=1)
    else:
        n, a, b = graphs.sbm(1_000_000, 1000, 2.1, 12.0, 2.0, seed=1)
    r = 10.0 * np.sqrt(n)
    pos = graphs.uniform_positions(n, -r, r, seed=2)
    return n, a, b, pos


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """SM clock and clock-event (throttle) reasons sampled while the timed
    region runs: NVML read every 5 ms from a host thread (a 50-iteration
    region lasts ~50 ms), else `nvidia-smi -lms 200`. Only reads the GPU's
    state. `__enter__` returns once the first sample is in, so the samples
    cover the region that follows."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReasons bits (nvml.h): SW power cap, HW slowdown, SW
    # thermal, HW thermal
    NVML_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8,
                 "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}
    NVML_CLOCK_SM = 1

    def __init__(self, device: int):
        self.dev = device
        self.proc = None
        self.f = None
        self.nvml = None
        self.handle = None
        self.rows = []
        self.stop = None
        self.thread = None
        self.source = None

    def _nvml_handle(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return False
        except Exception:
            return False
        h = C.c_void_p()
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.dev)
            bus = f"{pr.pci_domain_id:08x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
            rc = lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), C.byref(h))
        except Exception:
            rc = -1
        if rc != 0:
            visible = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            if visible and "," not in visible and visible.strip().isdigit():
                idx = int(visible)
            else:
                idx = self.dev
            if lib.nvmlDeviceGetHandleByIndex_v2(idx, C.byref(h)) != 0:
                return False
        self.nvml, self.handle = lib, h
        return True

    def _nvml_loop(self):
        import ctypes as C
        lib, h = self.nvml, self.handle
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        mx = C.c_uint(0)
        lib.nvmlDeviceGetMaxClockInfo(h, self.NVML_CLOCK_SM, C.byref(mx))
        while True:
            mhz = C.c_uint(0)
            why = C.c_ulonglong(0)
            if lib.nvmlDeviceGetClockInfo(h, self.NVML_CLOCK_SM, C.byref(mhz)) == 0 and \
                    get_reasons(h, C.byref(why)) == 0:
                r = [name for name, bit in self.NVML_BITS.items() if why.value & bit]
                self.rows.append((float(mhz.value), float(mx.value), r))
            if self.stop.wait(0.005):
                break

    def __enter__(self):
        import threading
        try:
            if self._nvml_handle():
                self.source = "nvml, every 5 ms"
                self.stop = threading.Event()
                self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
                self.thread.start()
                t0 = time.time()
                while not self.rows and time.time() - t0 < 1.0:
                    time.sleep(0.001)
                return self
        except Exception:
            self.thread = None
        try:
            self.source = "nvidia-smi -lms 200"
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 3.0 and os.path.getsize(self.f.name) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.thread:
            self.stop.set()
            self.thread.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def _smi_rows(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        rows = []
        self.f.flush()
        with open(self.f.name) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 8:
                    continue
                try:
                    rows.append((float(p[0]), float(p[1]),
                                 [names[k] for k in range(4)
                                  if p[4 + k].lower().startswith("active")]))
                except ValueError:
                    continue
        os.unlink(self.f.name)
        return rows

    def summary(self):
        if self.thread:
            rows = self.rows
        elif self.proc and self.f:
            rows = self._smi_rows()
        else:
            rows = []
            if self.f:
                os.unlink(self.f.name)
                self.f = None
        if not rows:
            return None
        reasons = sorted({x for _, _, r in rows for x in r})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "source": self.source}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def spawn_pool():
    """Worker processes for graph generation (spawned, never forked: a fork
    after the first CUDA call can hang)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    workers = max(1, min(16, (os.cpu_count() or 2) - 1))
    return ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"))


def _timed(stream, fn):
    """CUDA-event milliseconds of fn() on `stream` (a torch stream)."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def _rel_err(a, b):
    den = np.sqrt((b ** 2).sum(1)).max()
    return float(np.sqrt(((a - b) ** 2).sum(1)).max() / den)


def _pinned(arr):
    import torch
    t = torch.empty(arr.shape, dtype=getattr(torch, str(arr.dtype)), pin_memory=True)
    out = t.numpy()
    out[...] = arr
    return out, t


def full_run_e2e(g, pos, iters, local, calls=2, linlog=False, outbound=False):
    """node-iterations/s of fa2_full_run (the package's C call) from pinned
    host buffers: uploads, `iters` iterations and the download of the
    positions, `calls` timed calls after one warm-up call."""
    import ctypes as C
    from forceatlas2_rc_gb300 import _lib
    from forceatlas2_rc_gb300._abi import FA2_FULL_NTIMES, dptr
    from forceatlas2_rc_gb300.layout import Graph, _params
    n = g.n
    keep, host = [], {}
    for k, arr in (("inc_off", g.inc_off), ("inc_node", g.inc_node),
                   ("inc_coef", g.inc_coef), ("mass", g.mass),
                   ("size", np.ones(n)), ("fixed", np.zeros(n, np.int32)),
                   ("pos", np.ascontiguousarray(pos.T.reshape(-1)))):
        host[k], t = _pinned(np.ascontiguousarray(arr))
        keep.append(t)
    g2 = Graph.__new__(Graph)
    g2.n, g2.mass = n, host["mass"]
    g2.inc_off, g2.inc_node, g2.inc_coef = host["inc_off"], host["inc_node"], host["inc_coef"]
    p, keep2 = _params(g2, host["size"], host["fixed"], 2.0, 1.0, 1.2, 1.0, False, linlog,
                       False, iters, local, False)
    times = np.zeros(FA2_FULL_NTIMES)
    lib = _lib.load()
    xy0 = host["pos"].copy()
    h2d = sum(host[k].nbytes for k in ("inc_off", "inc_node", "inc_coef", "mass", "pos"))
    d2h = host["pos"].nbytes
    host["pos"][:] = xy0
    assert lib.fa2_full_run(C.byref(p), dptr(host["pos"]), dptr(times)) == 0, _lib.error()
    t0 = time.perf_counter()
    for _ in range(calls):
        host["pos"][:] = xy0
        assert lib.fa2_full_run(C.byref(p), dptr(host["pos"]), dptr(times)) == 0, _lib.error()
    dt = time.perf_counter() - t0
    return {"value": n * iters * calls / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "step": f"fa2_full_run, {iters} iterations, host buffers (pinned)",
            "s_per_layout": dt / calls}


# ---- the CPU legs: the reference's engine on the host cores ----------------

def cpu_engine():
    """Which build of the reference's CPU engine this host can run:
    "reference", the package's own src/forceatlas2.c compiled from its
    sources (oracle/_ref, where it was built for this machine), else "port",
    the oracle's restatement (bit-identical to it on every golden case)."""
    import oracle
    try:
        if oracle.ref_lib() is not None:
            return "reference"
    except OSError:  # built for another machine
        pass
    return "port"


def cpu_sample(n, a, b, w, pos, iters, threads, linlog, outbound):
    """The reference's CPU engine (C_forceatlas2 with the Gephi quadtree) on
    this host: node-iterations/s over `iters` iterations after one warm-up
    iteration, and which build ran (cpu_engine)."""
    import oracle
    kind = cpu_engine()
    which = "ref" if kind == "reference" else "oracle"
    o = oracle.Opts(scaling=2.0, gravity=1.0, linlog=linlog, outbound=outbound,
                    barnes_hut=True, theta=1.2, threads=threads)
    p1 = oracle.layout(n, a, b, w, pos, None, None, 1, o, which=which)
    t0 = time.perf_counter()
    oracle.layout(n, a, b, w, p1, None, None, iters, o, which=which)
    dt = time.perf_counter() - t0
    return n * iters / dt, dt, kind


def gpu_mode_leg(local):
    """The reference's `_gpu` mode (layout_forceatlas2_gpu): each iteration
    the caller builds the Gephi quadtree on the CPU (src/forceatlas2.c:698,
    here the oracle's restatement of tree_build, all host threads) and hands it to
    fa2_gpu_repulse_bh, this library's backend, which converts it on the
    device, walks it and adds the forces back (fa2_gpu_times: send, compute,
    fetch). Also the exact backend (fa2_gpu_repulse_exact) and the CPU's own
    Barnes-Hut repulsion on every host core. Config-2 graph, 100,000 nodes."""
    import ctypes as C
    import oracle
    from forceatlas2_rc_gb300 import _lib, graphs
    from forceatlas2_rc_gb300._abi import dptr
    lib = _lib.load()
    n, a, b = graphs.barabasi_albert(100_000, 3, seed=1)
    pos = graphs.uniform_positions(n, 0.0, 1000.0, seed=3)
    m, _ = oracle.mass(n, a, b)
    threads = os.cpu_count() or 1
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        qt = oracle.QuadTree(n, pos, m, threads=threads)
    tree_ms = 1000.0 * (time.perf_counter() - t0) / reps
    x, y = pos[:, 0].copy(), pos[:, 1].copy()
    out = {"n": n, "graph": "Barabasi-Albert m=3 (config 2), positions U[0,1000]^2",
           "tree_build_ms": tree_ms,
           "tree_build": f"oracle restatement of tree_build, {threads} threads (the "
                         f"regions of a level in parallel, as the reference)",
           "regions": int(qt.nreg)}
    t0 = time.perf_counter()
    oracle.repulse_bh(qt, pos, m, None, 0, 2.0, 1.2, threads=threads)
    out["cpu_repulse_bh_ms"] = 1000.0 * (time.perf_counter() - t0)
    out["cpu_threads"] = threads
    for use_double in (0, 1):
        h = lib.fa2_gpu_open(local, use_double, n, 0, 1, threads)
        assert h, _lib.error()
        dx, dy = np.zeros(n), np.zeros(n)
        assert lib.fa2_gpu_repulse_bh(h, C.byref(qt.t), 2.0, 1.2, dptr(dx), dptr(dy)) == 0, \
            _lib.error()
        t = np.zeros(3)
        lib.fa2_gpu_times(h, dptr(t))
        t0 = time.perf_counter()
        for _ in range(reps):
            assert lib.fa2_gpu_repulse_bh(h, C.byref(qt.t), 2.0, 1.2, dptr(dx), dptr(dy)) == 0
        wall = 1000.0 * (time.perf_counter() - t0) / reps
        t2 = np.zeros(3)
        lib.fa2_gpu_times(h, dptr(t2))
        d = (t2 - t) * 1000.0 / reps
        key = "repulse_bh_double" if use_double else "repulse_bh_single"
        out[key] = {"send_ms": d[0], "compute_ms": d[1], "fetch_ms": d[2], "call_ms": wall}
        lib.fa2_gpu_close(h)
    h = lib.fa2_gpu_open(local, 0, n, 0, 0, threads)
    assert h, _lib.error()
    dx, dy = np.zeros(n), np.zeros(n)
    assert lib.fa2_gpu_repulse_exact(h, dptr(x), dptr(y), dptr(m), None, 2.0, dptr(dx),
                                     dptr(dy)) == 0, _lib.error()
    t = np.zeros(3)
    lib.fa2_gpu_times(h, dptr(t))
    t0 = time.perf_counter()
    for _ in range(3):
        lib.fa2_gpu_repulse_exact(h, dptr(x), dptr(y), dptr(m), None, 2.0, dptr(dx), dptr(dy))
    wall = 1000.0 * (time.perf_counter() - t0) / 3
    t2 = np.zeros(3)
    lib.fa2_gpu_times(h, dptr(t2))
    d = (t2 - t) * 1000.0 / 3
    out["repulse_exact_single"] = {"send_ms": d[0], "compute_ms": d[1], "fetch_ms": d[2],
                                   "call_ms": wall}
    lib.fa2_gpu_close(h)
    bh = out["repulse_bh_single"]["call_ms"]
    out["gpu_mode_iteration_ms"] = tree_ms + bh
    out["cpu_tree_share_of_gpu_mode"] = tree_ms / (tree_ms + bh)
    return out


def cpu_legs(args, heads):
    """Every use of the oracle in the bench: the reference's CPU engine timed
    on the host's cores on bounded samples of each workload (the
    cpu_baseline objects), the host graph preparation of the package's .Call
    layer, and the reference's `_gpu` mode whose per-iteration quadtree is
    the reference's CPU code."""
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    out = {}
    n, a, b = heads["sbm"]
    r = 10.0 * np.sqrt(n)
    from forceatlas2_rc_gb300 import graphs
    pos = graphs.uniform_positions(n, -r, r, seed=2)
    iters = 10 if args.small else 40
    cv, cdt, kind = cpu_sample(n, a, b, np.ones(len(a)), pos, iters, threads, True, True)
    t0 = time.perf_counter()
    oracle.prepare_large(n, a, b, np.ones(len(a)), outbound=True)
    prep_s = time.perf_counter() - t0
    out["sbm"] = {"value": cv, "unit": UNIT, "cores": threads, "kind": kind,
                  "sample": f"{iters} iterations of the full {n}-node workload (after 1 "
                            f"warm-up), C_forceatlas2 quadtree engine, {cdt:.1f} s",
                  "graph_prep_s": prep_s,
                  "graph_prep": "C_forceatlas2_large's host preparation (masses, incidence "
                                "lists), oracle restatement, 1 core"}
    if "ba" in heads:
        n, a, b, w, pos = heads["ba"]
        cv, cdt, kind = cpu_sample(n, a, b, w, pos, 50, threads, False, False)
        out["ba"] = {"value": cv, "unit": UNIT, "cores": threads, "kind": kind,
                     "sample": f"50 iterations of the {n}-node workload (after 1 warm-up), "
                               f"C_forceatlas2 quadtree engine, {cdt:.1f} s"}
    if heads.get("gpu_mode"):
        try:
            out["gpu_mode"] = gpu_mode_leg(heads["local"])
        except Exception as e:  # reported, never fatal to the headline
            out["gpu_mode"] = {"error": repr(e)[:300]}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    kind = cpu_engine()
    which = "ref" if kind == "reference" else "oracle"
    n, a, b, _ = make_workload(args.small)
    w = np.ones(len(a))
    o = oracle.Opts(scaling=2.0, gravity=1.0, linlog=True, outbound=True,
                    barnes_hut=True, theta=1.2, threads=threads)
    r = 10.0 * np.sqrt(n)
    from forceatlas2_rc_gb300 import graphs
    pos = graphs.uniform_positions(n, -r, r, seed=2)
    pos = oracle.layout(n, a, b, w, pos, None, None, args.warmup, o, which=which)
    t0 = time.perf_counter()
    oracle.layout(n, a, b, w, pos, None, None, args.steps, o, which=which)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "edges": int(len(a)),
                   "engine": "src/forceatlas2.c C_forceatlas2 loop (quadtree "
                             "Barnes-Hut, OpenMP), " +
                             ("compiled from the reference's sources" if kind == "reference"
                              else "oracle restatement")},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": kind,
                         "sample": f"{args.steps} iterations of the full "
                                   f"workload after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_exact(args):
    """The all-pairs repulsion kernel alone (fa2_gpu_repulse_exact's
    kernel, through a resident exact layout): 100,000 nodes, FP32, pairs/s
    and the FP32-pipe rate it implies (20 FLOP per pair, the n-body
    convention)."""
    from forceatlas2_rc_gb300 import graphs
    from forceatlas2_rc_gb300.layout import REPULSION_EXACT, Graph, Layout
    n = 20_000 if args.small else 100_000
    e = np.zeros(0, np.int32)
    g = Graph(n, e, e, np.zeros(0))
    pos = graphs.uniform_positions(n, -1000.0, 1000.0, seed=3)
    L = Layout(g, pos, precision="single", repulsion=REPULSION_EXACT,
               scaling=2.0, gravity=1.0)
    L.iterate(max(args.warmup, 1))
    L.sync()
    if args.profile_only:
        L.close()
        return 0
    reps = max(3, args.steps // 10)
    ph = L.phase_times(reps)
    ms = ph["repulsion"] / reps
    pairs = float(n) * n
    tflops = 20.0 * pairs / (ms / 1000.0) / 1e12
    print(json.dumps({"workload": f"exact all-pairs repulsion, n={n}, FP32",
                      "kernel": "k_exact<float, 0, 4> (+ k_pack, k_exact_sum)",
                      "launch_ms": ms,
                      "pairs_per_s": pairs / (ms / 1000.0),
                      "fp32_tflops_20flop_convention": tflops,
                      "n": n}), flush=True)
    L.close()
    return 0


# ---- config 2: Barabasi-Albert, 100,000 nodes ---------------------------------

BA_WORKLOAD = ("Barabasi-Albert n=100,000, m=3 (~300k edges), weights lognormal(0, 0.5), "
               "positions U[0,1000]^2; Barnes-Hut theta 1.2 on the Morton/Karras pipeline, "
               "FP32 positions/forces, FP64 swing/traction totals and speed control, "
               "scaling 2, gravity 1, 500 iterations")


def ba_workload(small=False):
    from forceatlas2_rc_gb300 import graphs
    n, a, b = graphs.barabasi_albert(20_000 if small else 100_000, 3, seed=1)
    w = np.random.default_rng(1).lognormal(0.0, 0.5, len(a))
    pos = graphs.uniform_positions(n, 0.0, 1000.0, seed=3)
    return n, a, b, w, pos


def ba_result(args, local, work):
    """Config 2 through the resident layout: FP32 and same-GPU FP64
    node-iterations/s over one 500-iteration layout each, the per-step force
    error of FP32 against FP64 (the FP64 path equals the oracle's double
    construction bit for bit) at the start and at the end, phase times, and
    the layout end to end through fa2_full_run."""
    import torch
    from forceatlas2_rc_gb300.layout import REPULSION_BH, Graph, Layout
    n, a, b, w, pos = work
    iters = 500
    g = Graph(n, a, b, w)
    kw = dict(scaling=2.0, gravity=1.0, theta=1.2, device=local)
    out = {"workload": BA_WORKLOAD, "n": n, "edges": int(len(a)), "iterations": iters}
    L = Layout(g, pos, precision="single", repulsion=REPULSION_BH, **kw)
    # kernels of one captured iteration (fa2cu_layout_info)
    out["launches_per_iteration"] = int(L.info("launches_per_iteration"))
    # force errors from identical positions: coordinates the FP32 path holds
    pos32 = pos.astype(np.float32).astype(np.float64)
    f0_32 = L.forces(pos32)
    L.set_positions(pos)
    L.iterate(max(args.warmup, 3))
    L.set_positions(pos)
    L.sync()
    st = torch.cuda.ExternalStream(L.stream, device=local)
    with Clocks(local) as clk:
        ms = _timed(st, lambda: L.iterate(iters))
    L.sync()
    xy = L.positions()
    f1_32 = L.forces(xy)
    ph = L.phase_times(10)
    L.close()
    L64 = Layout(g, pos, precision="double", repulsion=REPULSION_BH, **kw)
    f0_64 = L64.forces(pos32)
    f1_64 = L64.forces(xy)
    L64.set_positions(pos)
    L64.iterate(3)
    L64.set_positions(pos)
    L64.sync()
    st64 = torch.cuda.ExternalStream(L64.stream, device=local)
    ms64 = _timed(st64, lambda: L64.iterate(iters))
    L64.sync()
    L64.close()
    out.update({
        "value": n * iters / (ms / 1000.0), "unit": UNIT, "iterations_per_s": iters / (ms / 1000.0),
        "ms_per_layout": ms,
        "fp64_value": n * iters / (ms64 / 1000.0),
        "fp32_over_fp64": ms64 / ms,
        "force_err_fp32_vs_fp64_start": _rel_err(f0_32, f0_64),
        "force_err_fp32_vs_fp64_end": _rel_err(f1_32, f1_64),
        "phase_ms": {k: v / 10.0 for k, v in ph.items()},
        "clocks": clk.summary(),
        "l2": "working set ~30 MB fits in L2: timed as resident iterations, no flush",
    })
    if not args.no_e2e:
        out["e2e"] = full_run_e2e(g, pos, iters, local)
    return out


def run_ba(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    from forceatlas2_rc_gb300 import build as fbuild
    fbuild.build()
    work = ba_workload(args.small)
    r = ba_result(args, local, work)
    cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        n, a, b, w, pos = work
        cv, cdt, kind = cpu_sample(n, a, b, w, pos, 50, os.cpu_count() or 1, False, False)
        cpu = {"value": cv, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": kind,
               "sample": f"50 iterations (after 1 warm-up), C_forceatlas2 quadtree "
                         f"engine, {cdt:.1f} s"}
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1,
            "steps": r["iterations"], "warmup": max(args.warmup, 3),
            "ms_per_step": r["ms_per_layout"] / r["iterations"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BA_WORKLOAD, "n": r["n"], "edges": r["edges"]},
            "result": r, "e2e": r.get("e2e"), "cpu_baseline": cpu,
            "gpu_launches": r["launches_per_iteration"] * r["iterations"],
            "clocks": r["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---- config 4: many small graphs in one persistent launch ---------------------

BATCH_WORKLOAD = ("4096 independent graphs, alternately Erdos-Renyi and "
                  "islands of 40 nodes, sizes log-uniform in [50, 20000], mean "
                  "degree uniform in [4, 16] per graph, unit weights; scaling 2, "
                  "gravity 1, theta 1.2; exact repulsion below the autotuned "
                  "crossover, Barnes-Hut above; FP32 with per-graph FP64 speed "
                  "state; 500 iterations each")


def batch_plan(count: int, seed: int = 11):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(50.0), np.log(20000.0), count)).astype(int)
    degs = rng.uniform(4.0, 16.0, count)
    return [(i, int(sizes[i]), float(degs[i])) for i in range(count)]


def batch_graphs(items):
    """Graphs and start positions of the batch items (i, n, mean degree)."""
    from forceatlas2_rc_gb300 import graphs
    from forceatlas2_rc_gb300.layout import Graph
    out = []
    for i, n, deg in items:
        gen = graphs.erdos_renyi if i % 2 == 0 else graphs.island_graph
        _, a, b = gen(n, deg, seed=100 + i)
        r = 10.0 * np.sqrt(n)
        out.append((Graph(n, a, b, np.ones(len(a))),
                    graphs.uniform_positions(n, -r, r, seed=5000 + i)))
    return out


def batch_workload(count: int, pool=None):
    plan = batch_plan(count)
    chunks = [plan[k:k + 64] for k in range(0, len(plan), 64)]
    res = pool.map(batch_graphs, chunks) if pool else map(batch_graphs, chunks)
    gs, ps = [], []
    for part in res:
        for g, p in part:
            gs.append(g)
            ps.append(p)
    return gs, ps


def batch_result(args, local, work, full=False):
    """Config 4: layouts/s of the batched engine (one persistent launch,
    CUDA-graph replayed, graphs resident) against the single-graph engine
    called once per graph on the same GPU; e2e with the uploads and
    downloads of every graph."""
    import torch
    from forceatlas2_rc_gb300.batch import Batch, tune
    from forceatlas2_rc_gb300.layout import REPULSION_BH, REPULSION_EXACT, Layout
    gs, ps = work
    count = len(gs)
    iters = 100 if args.small else 500
    nodes = sum(g.n for g in gs)
    t0 = time.perf_counter()
    tuned = tune(local, "single")
    tune_s = time.perf_counter() - t0
    kw = dict(scaling=2.0, gravity=1.0, theta=1.2)
    # e2e: upload of every graph, the layout, download of every graph (this
    # pass also captures the launch that the timed steps replay)
    t0 = time.perf_counter()
    B = Batch(gs, ps, precision="single", device=local, **kw)
    B.iterate(iters)
    B.sync()
    out = [B.positions(i) for i in range(count)]
    e2e_s = time.perf_counter() - t0
    h2d = sum(g.inc_off.nbytes + g.inc_node.nbytes + g.inc_coef.nbytes +
              g.mass.nbytes + 16 * g.n for g in gs)
    d2h = sum(16 * g.n for g in gs)
    assert all(np.isfinite(o).all() for o in out)
    stream = torch.cuda.ExternalStream(B.stream, device=local)
    steps = max(1, min(args.steps, 3 if full else 1))
    for _ in range(max(args.warmup, 1) if full else 0):
        B.iterate(iters)
    B.sync()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        ms = _timed(stream, lambda: [B.iterate(iters) for _ in range(steps)])
    B.sync()
    B.close()
    value = count * steps / (ms / 1000.0)
    # the single-graph engine, one graph at a time (open, iterate, fetch,
    # close), on an evenly spaced sample of the graphs
    pick = list(range(0, count, max(1, count // 64)))
    t0 = time.perf_counter()
    for i in pick:
        rep = REPULSION_EXACT if gs[i].n < tuned["exact_below"] else REPULSION_BH
        with Layout(gs[i], ps[i], precision="single", repulsion=rep, device=local, **kw) as L:
            L.iterate(iters)
            L.sync()
            L.positions()
    loop_s = time.perf_counter() - t0
    loop_value = len(pick) / loop_s
    loop_nodes = sum(gs[i].n for i in pick)
    # per-step force error of the batched engine, FP32 against FP64, on the
    # same sample (one iteration from identical float-representable
    # positions, the forces the batch kept: fa2cu_batch_forces)
    sub_g = [gs[i] for i in pick]
    sub_p = [np.asarray(ps[i]).astype(np.float32).astype(np.float64) for i in pick]
    fe = {}
    for prec in ("single", "double"):
        with Batch(sub_g, sub_p, precision=prec, device=local,
                   exact_below=tuned["exact_below"], threads=tuned["threads"],
                   nodes_per_thread=tuned["nodes_per_thread"], **kw) as Bf:
            Bf.iterate(1)
            Bf.sync()
            fe[prec] = [Bf.forces(k) for k in range(len(sub_g))]
    errs = [_rel_err(a, b) for a, b in zip(fe["single"], fe["double"])]
    return {
        "workload": BATCH_WORKLOAD if not args.small else f"{count} graphs (small check)",
        "value": value, "unit": "layouts/s", "steps": steps, "ms_per_step": ms / steps,
        "graphs": count, "nodes": nodes, "iterations": iters,
        "exact_below": tuned["exact_below"], "threads": tuned["threads"],
        "nodes_per_thread": tuned["nodes_per_thread"],
        "node_iters_per_s": nodes * iters * steps / (ms / 1000.0),
        "e2e": {"value": count / e2e_s, "unit": "layouts/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step": f"Batch open (upload) + {iters} iterations + positions of every graph"},
        "one_graph_at_a_time": {
            "value": loop_value, "unit": "layouts/s",
            "sample": f"{len(pick)} of the {count} graphs ({loop_nodes} nodes), "
                      f"fa2cu_layout open/iterate/positions/close each, {loop_s:.1f} s",
            "node_iters_per_s": loop_nodes * iters / loop_s},
        "batched_over_loop": value / loop_value,
        "batched_e2e_over_loop": (count / e2e_s) / loop_value,
        "force_err_fp32_vs_fp64": max(errs),
        "force_err_fp32_vs_fp64_median": float(np.median(errs)),
        "force_err_sample": f"the batched engine's forces of one iteration, FP32 against "
                            f"FP64 from identical positions, on the {len(pick)} graphs of "
                            f"the loop's sample (largest and median of the per-graph "
                            f"norm-wise errors)",
        "gpu_launches": steps, "autotune_s": tune_s,
        "l2": "working set > 129 MB L2 (no flush needed)",
        "clocks": clk.summary(),
    }


def run_batch(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    count = 256 if args.small else 4096
    t0 = time.perf_counter()
    with spawn_pool() as pool:
        work = batch_workload(count, pool)
    gen_s = time.perf_counter() - t0
    r = batch_result(args, local, work, full=True)
    line = {"metric": "layouts/s (batched, 500 iterations each)", "value": r["value"],
            "unit": "layouts/s", "n_gpus": 1, "steps": r["steps"],
            "warmup": max(args.warmup, 1), "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": r["workload"], "graphs": r["graphs"], "nodes": r["nodes"],
                       "iterations": r["iterations"], "exact_below": r["exact_below"],
                       "threads": r["threads"], "l2": r["l2"]},
            "result": r, "e2e": r["e2e"], "gpu_launches": r["gpu_launches"],
            "generate_s": gen_s, "clocks": r["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---- config 5: the layout server on a Poisson job trace -----------------------

SERVE_WORKLOAD = ("layout jobs with Poisson arrivals at 200 requests/s; sizes "
                  "log-uniform in [1000, 2000000] nodes, drawn per job; 50/50 "
                  "Barabasi-Albert (m in 2..5) and SBM (blocks of ~1000 nodes, "
                  "power-law sizes, deg_in 12, deg_out 2); 30% continuations from "
                  "stored coordinates with prevent_overlap and node_size U[1,5]; "
                  "10% pin their top-1% degree nodes; iterations U[200,1000]; FP32 "
                  "Barnes-Hut theta 1.2, scaling 2, gravity 1")


def serve_trace(count: int, rate: float, seed: int = 5):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    jobs = []
    for i in range(count):
        kind = "ba" if rng.random() < 0.5 else "sbm"
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e6))))
        jobs.append(dict(t=float(t[i]), kind=kind, n=n, m=int(rng.integers(2, 6)),
                         cont=bool(rng.random() < 0.3), pin=bool(rng.random() < 0.1),
                         iters=int(rng.integers(200, 1001)), seed=1000 + i))
    return jobs


def serve_graph(job):
    """A job's graph (generated per job, at its own size)."""
    from forceatlas2_rc_gb300 import graphs
    from forceatlas2_rc_gb300.layout import Graph
    n = job["n"]
    if job["kind"] == "ba":
        _, a, b = graphs.barabasi_albert_fast(n, job["m"], seed=job["seed"])
    else:
        _, a, b = graphs.sbm(n, max(2, n // 1000), 2.1, 12.0, 2.0, seed=job["seed"])
    return Graph(n, a, b, np.ones(len(a)))


def serve_inputs(jobs, gs, local):
    """Every job's start positions and settings, made before the clock
    starts; a continuation starts from stored coordinates (its graph after
    30 iterations from random positions)."""
    from forceatlas2_rc_gb300 import graphs
    from forceatlas2_rc_gb300.layout import Layout
    out = []
    for j, g in zip(jobs, gs):
        rng = np.random.default_rng(j["seed"])
        r = 10.0 * np.sqrt(g.n)
        kw = dict(scaling=2.0, gravity=1.0, theta=1.2)
        pos = graphs.uniform_positions(g.n, -r, r, seed=j["seed"])
        if j["cont"]:
            with Layout(g, pos, device=local, **kw) as L:
                L.iterate(30)
                L.sync()
                pos = L.positions()
            kw.update(adjust=True, size=rng.uniform(1.0, 5.0, g.n))
        if j["pin"]:
            deg = g.mass - 1.0
            top = np.argsort(-deg, kind="stable")[:max(1, g.n // 100)]
            fixed = np.zeros(g.n, np.int32)
            fixed[top] = 1
            kw["fixed"] = fixed
        out.append(dict(g=g, pos=pos, kw=kw))
    return out


def serve_pass(jobs, inputs, times, device, max_jobs, policy="arrival"):
    """Submit the jobs at their arrival times (seconds from the start) to a
    fresh server, collect every result on another thread; latency = end -
    arrival."""
    import threading
    from forceatlas2_rc_gb300 import _lib
    from forceatlas2_rc_gb300.serve import Server
    lib = _lib.load()
    done = []
    submitted = threading.Semaphore(0)
    with Server(device=device, max_jobs=max_jobs, chunk=16, policy=policy) as S:
        def collect():
            for _ in range(len(jobs)):
                submitted.acquire()  # a job to wait for
                r = S.wait()
                done.append((r[0], r[2]))
        th = threading.Thread(target=collect)
        th.start()
        arrival = {}
        t0 = time.perf_counter()
        c0 = lib.fa2_now()
        for j, inp, ta in zip(jobs, inputs, times):
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            jid = S.submit(inp["g"], inp["pos"], j["iters"], **inp["kw"])
            arrival[jid] = ta
            submitted.release()
        th.join()
        st = S.stats()
    lat = np.array([m["t_end"] - (c0 + arrival[jid]) for jid, m in done])
    queued = np.array([m["t_resident"] - m["t_submit"] for _, m in done])
    end = max(m["t_end"] for _, m in done) - c0
    node_iters = sum(m["n"] * m["iterations"] for _, m in done)
    span = times[-1] - times[0] if len(times) > 1 else 0.0
    return {"jobs": len(done), "makespan_s": end,
            "layouts_per_s": len(done) / end,
            "node_iters_per_s": node_iters / end,
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()),
            "p50_wait_resident_s": float(np.percentile(queued, 50)),
            "peak_footprint_gb": st["peak_footprint"] / 1e9,
            "pool_reserved_gb": st["pool_reserved"] / 1e9,
            "offered_rate_per_s": (len(times) - 1) / span if span > 0 else None,
            "max_jobs": max_jobs, "policy": policy}


def serve_workload(count, pool=None):
    jobs = serve_trace(count, 200.0)
    gs = list(pool.map(serve_graph, jobs)) if pool else [serve_graph(j) for j in jobs]
    return jobs, gs


def serve_result(args, local, work, full=False):
    """Config 5: continuous batching by the layout server. The trace at 200
    requests/s (far beyond what one GPU serves: the latencies are queueing),
    then the same kind of trace at 0.8 x the capacity measured on the first
    pass (a sustainable load); with `full`, also the 200/s trace admitted
    least work first and one job at a time."""
    jobs, gs = work
    t0 = time.perf_counter()
    inputs = serve_inputs(jobs, gs, local)
    prep_s = time.perf_counter() - t0
    # resident jobs: large jobs fill the GPU alone, and more of them at once
    # only share its caches
    resident = 4
    times = [j["t"] for j in jobs]
    with Clocks(local) as clk:
        busy = serve_pass(jobs, inputs, times, local, resident)
    cap = busy["layouts_per_s"]
    # the sustainable pass: the first jobs re-timed as Poisson arrivals at
    # 0.8 x capacity
    k = max(8, len(jobs) // 2)
    rng = np.random.default_rng(9)
    t_sus = list(np.cumsum(rng.exponential(1.0 / (0.8 * cap), k)))
    sus = serve_pass(jobs[:k], inputs[:k], t_sus, local, resident)
    out = {"workload": SERVE_WORKLOAD, "jobs": len(jobs),
           "nodes": [int(g.n) for g in gs],
           "value": busy["layouts_per_s"], "unit": "layouts/s",
           "p50_latency_s": busy["p50_latency_s"], "p99_latency_s": busy["p99_latency_s"],
           "at_200_per_s": busy, "at_0.8_capacity": sus,
           "prep_s": prep_s, "clocks": clk.summary(),
           "e2e": {"value": busy["layouts_per_s"], "unit": "layouts/s",
                   "h2d_bytes_per_step": int(np.mean([
                       i["g"].inc_off.nbytes + i["g"].inc_node.nbytes +
                       i["g"].inc_coef.nbytes + 32 * i["g"].n for i in inputs])),
                   "d2h_bytes_per_step": int(np.mean([16 * i["g"].n for i in inputs])),
                   "step": "one job: submit (host arrays) to collected positions"}}
    # per-step force error of the served layouts (the server runs Layout
    # sessions), FP32 against FP64 from identical positions, on the first
    # Barabasi-Albert and the first SBM job of the trace with their settings
    from forceatlas2_rc_gb300.layout import Layout
    ferr = {}
    for kind in ("ba", "sbm"):
        i = next((k for k, j in enumerate(jobs) if j["kind"] == kind), None)
        if i is None:
            continue
        inp = inputs[i]
        pos32 = np.asarray(inp["pos"]).astype(np.float32).astype(np.float64)
        fs = {}
        for prec in ("single", "double"):
            with Layout(inp["g"], pos32, precision=prec, device=local, **inp["kw"]) as L:
                fs[prec] = L.forces(pos32)
        ferr[f"{kind} n={inp['g'].n}"] = _rel_err(fs["single"], fs["double"])
    out["force_err_fp32_vs_fp64"] = max(ferr.values()) if ferr else None
    out["force_err_jobs"] = ferr
    if full:
        out["at_200_per_s_least_work_first"] = serve_pass(jobs, inputs, times, local,
                                                          resident, "least_work")
        out["one_job_at_a_time"] = serve_pass(jobs, inputs, times, local, 1)
    return out


def run_serve(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    count = 24 if args.small else 64
    t0 = time.perf_counter()
    with spawn_pool() as pool:
        work = serve_workload(count, pool)
    gen_s = time.perf_counter() - t0
    r = serve_result(args, local, work, full=True)
    line = {"metric": "served layouts/s, p50/p99 latency", "value": r["value"],
            "unit": "layouts/s", "n_gpus": 1, "steps": r["jobs"], "warmup": 0,
            "ms_per_step": 1000.0 * r["at_200_per_s"]["makespan_s"] / r["jobs"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": SERVE_WORKLOAD, "jobs": r["jobs"],
                       "l2": "working sets > 129 MB L2 for the large jobs"},
            "p50_latency_s": r["p50_latency_s"], "p99_latency_s": r["p99_latency_s"],
            "result": r, "e2e": r["e2e"], "generate_s": gen_s, "clocks": r["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---- the headline line (config 3) with the other configs beside it -------------

def headline(args, local, ws, pg):
    import torch
    from forceatlas2_rc_gb300 import _lib
    from forceatlas2_rc_gb300._abi import FA2_FULL_NTIMES, dptr
    from forceatlas2_rc_gb300.layout import REPULSION_BH, Graph, Layout, _params

    n, a, b, pos = make_workload(args.small)
    g = Graph(n, a, b, np.ones(len(a)), outbound=True)
    kw = dict(scaling=2.0, gravity=1.0, theta=1.2, linlog=True, device=local)
    L = Layout(g, pos, precision="single", repulsion=REPULSION_BH, **kw)
    L.option("walk", WALKS[args.walk])
    stream = torch.cuda.ExternalStream(L.stream, device=local)
    # kernels of one captured iteration: Morton codes (with the sort's digit
    # histograms), 4 sort passes, gather + Karras tree, the bottom-up sums,
    # the traversal; beside the tree and the traversal on a second stream,
    # (the hubs' attraction, if any) gravity and attraction; then the join
    # with the swing totals and the speed update, the displacement (with the
    # next bounding box); no memset
    launches = int(L.info("launches_per_iteration"))

    if args.profile_only:
        L.iterate(max(args.warmup, 1))
        L.sync()
        L.close()
        return None

    L.iterate(args.warmup)
    L.sync()

    # ---- value: device-resident throughput --------------------------------
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        ms = _timed(stream, lambda: L.iterate(args.steps))
    L.sync()
    torch.cuda.synchronize()
    if pg:
        t = torch.tensor([ms], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
        pg.barrier()
    clocks = clk.summary()
    value = ws * n * args.steps / (ms / 1000.0)

    # ---- phase times (CUDA events on the layout's stream) -----------------
    ph = L.phase_times(10)
    ph = {k: v / 10.0 for k, v in ph.items()}
    counts = L.traversal_counts()

    # ---- FP32 vs FP64: force error and same-GPU FP64 throughput (from
    #      identical positions: coordinates the FP32 path holds) -------------
    pos32 = pos.astype(np.float32).astype(np.float64)
    f0_32 = L.forces(pos32)
    xy = L.positions()
    f32 = L.forces(xy)
    L.close()
    L64 = Layout(g, xy, precision="double", repulsion=REPULSION_BH, **kw)
    f64 = L64.forces(xy)
    f0_64 = L64.forces(pos32)
    force_err = _rel_err(f32, f64)
    L64.set_positions(xy)
    L64.iterate(2)
    L64.sync()
    k64 = max(3, args.steps // 10)
    s64 = torch.cuda.ExternalStream(L64.stream, device=local)
    fp64_value = n * k64 / (_timed(s64, lambda: L64.iterate(k64)) / 1000.0)
    L64.sync()
    L64.close()

    # ---- e2e: fa2_full_run (the C interface the package calls) with host
    #      buffers in pinned memory; each step = one whole layout of 1000
    #      iterations, uploads and download included -------------------------
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        e2e = full_run_e2e(g, pos, 1000, local, linlog=True)
        if pg:
            t = torch.tensor([e2e["s_per_layout"]], device=f"cuda:{local}")
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            e2e["s_per_layout"] = float(t.item())
            e2e["value"] = ws * n * 1000 / e2e["s_per_layout"]
        # the same layout from the edge list: fa2cu_full_run_edges prepares
        # masses and incidence lists on the device (the host's O(m)
        # preparation of C_forceatlas2_large moves into the timed call)
        from forceatlas2_rc_gb300._abi import iptr
        from forceatlas2_rc_gb300.layout import _EdgeOnly
        keep = []
        ea, t1 = _pinned(np.ascontiguousarray(a, dtype=np.int32))
        eb, t2 = _pinned(np.ascontiguousarray(b, dtype=np.int32))
        ew, t3 = _pinned(np.ones(len(a)))
        hp, t4 = _pinned(np.ascontiguousarray(pos.T.reshape(-1)))
        hs, t5 = _pinned(np.ones(n))
        hf, t6 = _pinned(np.zeros(n, np.int32))
        keep += [t1, t2, t3, t4, t5, t6]
        iters = 1000
        pe, keep3 = _params(_EdgeOnly(n), hs, hf, 2.0, 1.0, 1.2, 1.0, False, True, False,
                            iters, local, False)
        lib = _lib.load()
        times = np.zeros(FA2_FULL_NTIMES)
        xy0 = hp.copy()
        run_e = lambda: lib.fa2cu_full_run_edges(  # noqa: E731
            C.byref(pe), len(a), iptr(ea), iptr(eb), dptr(ew), 1, dptr(hp), dptr(times))
        hp[:] = xy0
        assert run_e() == 0, _lib.error()
        calls = 2
        t0 = time.perf_counter()
        for _ in range(calls):
            hp[:] = xy0
            assert run_e() == 0, _lib.error()
        dte = time.perf_counter() - t0
        if pg:
            t = torch.tensor([dte], device=f"cuda:{local}")
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            dte = float(t.item())
        e2e["from_edges"] = {
            "value": ws * n * iters * calls / dte, "unit": UNIT,
            "h2d_bytes_per_step": int(ea.nbytes + eb.nbytes + ew.nbytes + hp.nbytes),
            "d2h_bytes_per_step": int(hp.nbytes),
            "step": "fa2cu_full_run_edges (edge list in, graph prepared on "
                    "the device), 1000 iterations, host buffers (pinned)",
            "s_per_layout": dte / calls}

    # ---- roofline of the dominant kernel (the traversal) -------------------
    peaks, kind = measured_peaks()
    t_trav = ph["repulsion"] / 1000.0
    alg = TRAVERSE_HBM_BYTES_PER_NODE * n
    achieved = alg / t_trav / 1e9
    l2_bytes = (TRAVERSE_L2_BYTES_PER_VISIT * counts["visits"] +
                TRAVERSE_L2_BYTES_PER_PAIR * counts["pairs"])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "traffic": TRAVERSE_DRAM_BYTES.get(args.walk) if n == 1_000_000 else None,
                "issue_active": TRAVERSE_ISSUE_ACTIVE.get(args.walk),
                "l1_throughput": TRAVERSE_L1_THROUGHPUT.get(args.walk),
                "bound_note": "L1- and issue-bound (ncu: L1 throughput ~86 % of peak, issue "
                              "active ~76 %, 95 % L1 hits); the HBM fraction is small by "
                              "design",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                  "one traversal launch on this workload",
                "kernel": {"warp": "k_traverse_warp<float, 0>",
                           "thread": "k_traverse<float, 0, 8>",
                           "wide": "k_traverse<float, 0, 1>",
                           "pair": "k_traverse_multi<float, 0, 2>",
                           "quad": "k_traverse_multi<float, 0, 4>",
                           "deferred": "k_traverse_deferred<float, 0, 8>"}[args.walk],
                "peak_kind": f"{kind} (HBM copy)",
                "launch_ms": ph["repulsion"],
                "l2_request_bytes": l2_bytes,
                "l2_request_gbs": l2_bytes / t_trav / 1e9,
                "visits_per_node": counts["visits"] / n,
                "pairs_per_node": counts["pairs"] / n}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "edges": int(len(a)),
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "working set > 129 MB L2 (no flush needed)",
                   "walk": args.walk},
        "fp64_value": fp64_value,
        "fp32_over_fp64": value / ws / fp64_value,
        "force_err_fp32_vs_fp64": force_err,
        "force_err_fp32_vs_fp64_start": _rel_err(f0_32, f0_64),
        "iterations_per_s": 1000.0 * args.steps / ms,
        "phase_ms": ph,
        "phase_note": ("CUDA events around each phase, its kernels run one after the "
                       "other; in the captured iteration the attraction runs beside the "
                       "climb and the traversal, so the phases add up to more than "
                       "ms_per_step"),
        "gpu_launches": launches * args.steps, "launches_per_iteration": launches,
        "e2e": e2e, "roofline": roofline, "cpu_baseline": None,
        "clocks": clocks,
    }
    return line, (n, a, b)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true",
                    help="small graphs (quick check, not a bench line)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="the headline line only (no config 2 / 4 / 5 / _gpu-mode objects)")
    ap.add_argument("--profile-only", action="store_true",
                    help="warm-up and a few iterations only (for ncu)")
    ap.add_argument("--workload", default="sbm1m",
                    choices=["sbm1m", "ba100k", "exact", "batch", "serve"],
                    help="sbm1m: the headline line (with configs 2, 4, 5 beside it); "
                         "ba100k: config 2 alone; exact: all-pairs repulsion "
                         "kernel alone on 100,000 nodes (FP32 pipe figures); "
                         "batch: 4096 graphs in one persistent launch; "
                         "serve: the layout server on a Poisson job trace")
    ap.add_argument("--walk", default="deferred",
                    choices=list(WALKS),
                    help="Barnes-Hut walk (the same interactions; deferred is the "
                         "FP32 default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "exact":
        return run_exact(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "ba100k":
        return run_ba(args)

    ws, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    from forceatlas2_rc_gb300 import build as fbuild
    fbuild.build()
    extras = not args.no_extras and ws == 1 and not args.profile_only
    pool = spawn_pool() if extras else None
    fut_batch = fut_serve = None
    if pool:
        # the other configs' graphs, generated on the host cores while the
        # GPU runs the headline
        plan = batch_plan(256 if args.small else 4096)
        fut_batch = [pool.submit(batch_graphs, plan[k:k + 64]) for k in range(0, len(plan), 64)]
        sjobs = serve_trace(24 if args.small else 64, 200.0)
        fut_serve = [pool.submit(serve_graph, j) for j in sjobs]
    t_start = time.perf_counter()
    res = headline(args, local, ws, pg)
    if res is None:
        if pool:
            pool.shutdown(cancel_futures=True)
        return 0
    line, sbm_graph = res
    heads = {"sbm": sbm_graph, "local": local}
    if extras:
        try:
            work = ba_workload(args.small)
            heads["ba"] = work
            line["ba100k"] = ba_result(args, local, work)
        except Exception as e:
            line["ba100k"] = {"error": repr(e)[:300]}
        try:
            gs, ps = [], []
            for f in fut_batch:
                for g, p in f.result():
                    gs.append(g)
                    ps.append(p)
            line["batch"] = batch_result(args, local, (gs, ps))
            del gs, ps
        except Exception as e:
            line["batch"] = {"error": repr(e)[:300]}
        try:
            line["serve"] = serve_result(args, local, (sjobs, [f.result() for f in fut_serve]))
        except Exception as e:
            line["serve"] = {"error": repr(e)[:300]}
        pool.shutdown()
        heads["gpu_mode"] = True
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_legs(args, heads)
        line["cpu_baseline"] = cpu["sbm"]
        if "ba" in cpu and isinstance(line.get("ba100k"), dict) and "value" in line["ba100k"]:
            line["ba100k"]["cpu_baseline"] = cpu["ba"]
        if "gpu_mode" in cpu:
            line["gpu_mode"] = cpu["gpu_mode"]
    line["wall_s"] = time.perf_counter() - t_start
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
