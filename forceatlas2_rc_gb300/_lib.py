"""Loader of libfa2cuda.so (the C interface of include/fa2.h and
include/fa2_cuda.h).

The library is built in-tree (``forceatlas2_rc_gb300/libfa2cuda.so``, see
build.py). There is no fallback: if the library is missing, loading fails
with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os

from ._abi import DevInfo, FullParams, ServerConfig, Tree

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfa2cuda.so")

_lib = None

P_D = C.POINTER(C.c_double)
P_I = C.POINTER(C.c_int)
P_U = C.POINTER(C.c_uint32)


def load(build_if_missing: bool = False):
    """The loaded library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from .build import build
            build()
        else:
            raise RuntimeError(
                "libfa2cuda.so is not built: run `python -m "
                "forceatlas2_rc_gb300.build` (needs nvcc)")
    lib = C.CDLL(LIB_PATH)
    sig = {
        "fa2_gpu_error": (C.c_char_p, []),
        "fa2_gpu_ndevices": (C.c_int, []),
        "fa2_gpu_device_info": (C.c_int, [C.c_int, C.POINTER(DevInfo)]),
        "fa2_gpu_open": (C.c_void_p, [C.c_int] * 6),
        "fa2_gpu_times": (None, [C.c_void_p, P_D]),
        "fa2_gpu_close": (None, [C.c_void_p]),
        "fa2_gpu_repulse_exact": (C.c_int, [C.c_void_p, P_D, P_D, P_D, P_D,
                                            C.c_double, P_D, P_D]),
        "fa2_gpu_repulse_bh": (C.c_int, [C.c_void_p, C.POINTER(Tree),
                                         C.c_double, C.c_double, P_D, P_D]),
        "fa2_gpu_shutdown": (None, []),
        "fa2_now": (C.c_double, []),
        "fa2_full_run": (C.c_int, [C.POINTER(FullParams), P_D, P_D]),
        "fa2cu_layout_open": (C.c_void_p, [C.POINTER(FullParams), P_D, C.c_int]),
        "fa2cu_layout_iterate": (C.c_int, [C.c_void_p, C.c_int]),
        "fa2cu_layout_sync": (C.c_int, [C.c_void_p]),
        "fa2cu_layout_positions": (C.c_int, [C.c_void_p, P_D]),
        "fa2cu_layout_set_positions": (C.c_int, [C.c_void_p, P_D]),
        "fa2cu_layout_forces": (C.c_int, [C.c_void_p, P_D, P_D]),
        "fa2cu_layout_speed": (C.c_int, [C.c_void_p, P_D]),
        "fa2cu_layout_stream": (C.c_void_p, [C.c_void_p]),
        "fa2cu_layout_phase_times": (C.c_int, [C.c_void_p, C.c_int, P_D]),
        "fa2cu_layout_tree": (C.c_int, [C.c_void_p, P_D, P_U, P_U, P_I, P_I,
                                        P_I, P_D]),
        "fa2cu_layout_traversal_counts": (C.c_int, [C.c_void_p, P_D]),
        "fa2cu_layout_option": (C.c_int, [C.c_void_p, C.c_char_p, C.c_double]),
        "fa2cu_layout_swing": (C.c_int, [C.c_void_p, P_D, P_D]),
        "fa2cu_layout_info": (C.c_double, [C.c_void_p, C.c_char_p]),
        "fa2cu_layout_bytes": (C.c_double, [C.c_void_p]),
        "fa2cu_layout_close": (None, [C.c_void_p]),
        "fa2cu_build_info": (C.c_char_p, []),
        "fa2cu_morton_order_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, C.c_void_p]),
        "fa2cu_noalloc_status": (C.c_int, [C.c_void_p]),
        "fa2cu_batch_open": (C.c_void_p, [C.POINTER(FullParams), C.c_int,
                                          C.POINTER(P_D), C.c_int, C.c_int,
                                          C.c_int]),
        "fa2cu_batch_iterate": (C.c_int, [C.c_void_p, C.c_int]),
        "fa2cu_batch_sync": (C.c_int, [C.c_void_p]),
        "fa2cu_batch_positions": (C.c_int, [C.c_void_p, C.c_int, P_D]),
        "fa2cu_batch_forces": (C.c_int, [C.c_void_p, C.c_int, P_D]),
        "fa2cu_batch_speed": (C.c_int, [C.c_void_p, C.c_int, P_D]),
        "fa2cu_batch_stream": (C.c_void_p, [C.c_void_p]),
        "fa2cu_batch_phase_cycles": (C.c_int, [C.c_void_p, C.c_int, P_D]),
        "fa2cu_batch_bytes": (C.c_double, [C.c_void_p]),
        "fa2cu_batch_close": (None, [C.c_void_p]),
        "fa2cu_batch_tune": (C.c_int, [C.c_int, C.c_int, P_I, P_I, P_I]),
        "fa2cu_server_open": (C.c_void_p, [C.POINTER(ServerConfig)]),
        "fa2cu_server_submit": (C.c_longlong, [C.c_void_p, C.POINTER(FullParams),
                                               P_D, C.c_int]),
        "fa2cu_server_wait": (C.c_longlong, [C.c_void_p, C.c_longlong, C.c_double,
                                             P_D]),
        "fa2cu_server_collect": (C.c_int, [C.c_void_p, C.c_longlong, P_D]),
        "fa2cu_server_stats": (C.c_int, [C.c_void_p, P_D]),
        "fa2cu_server_close": (None, [C.c_void_p]),
        "fa2cu_layout_footprint": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_int,
                                                C.c_int, C.c_int]),
        "fa2cu_graph_prep": (C.c_longlong, [C.c_int, C.c_int, C.c_int, P_I, P_I, P_D,
                                            C.c_int, P_D, P_I, P_I, P_D]),
        "fa2cu_layout_open_edges": (C.c_void_p, [C.POINTER(FullParams), C.c_int, P_I,
                                                 P_I, P_D, C.c_int, P_D, C.c_int]),
        "fa2cu_full_run_edges": (C.c_int, [C.POINTER(FullParams), C.c_int, P_I, P_I,
                                           P_D, C.c_int, P_D, P_D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def error() -> str:
    return load().fa2_gpu_error().decode(errors="replace")


# Entry points declared in include/*.h; the CPU tests check that the built
# library exports every one of them.
EXPORTED = (
    "fa2_gpu_error", "fa2_gpu_ndevices", "fa2_gpu_device_info",
    "fa2_gpu_open", "fa2_gpu_times", "fa2_gpu_close",
    "fa2_gpu_repulse_exact", "fa2_gpu_repulse_bh", "fa2_gpu_shutdown",
    "fa2_now", "fa2_full_run",
    "fa2cu_layout_open", "fa2cu_layout_iterate", "fa2cu_layout_sync",
    "fa2cu_layout_positions", "fa2cu_layout_set_positions",
    "fa2cu_layout_forces", "fa2cu_layout_speed", "fa2cu_layout_stream",
    "fa2cu_layout_phase_times", "fa2cu_layout_tree",
    "fa2cu_layout_traversal_counts", "fa2cu_layout_option", "fa2cu_layout_swing",
    "fa2cu_layout_info",
    "fa2cu_layout_bytes",
    "fa2cu_layout_close", "fa2cu_build_info", "fa2cu_morton_order_noalloc",
    "fa2cu_noalloc_status",
    "fa2cu_batch_open", "fa2cu_batch_iterate", "fa2cu_batch_sync", "fa2cu_batch_forces",
    "fa2cu_batch_positions", "fa2cu_batch_speed", "fa2cu_batch_stream",
    "fa2cu_batch_phase_cycles",
    "fa2cu_batch_bytes", "fa2cu_batch_close", "fa2cu_batch_tune",
    "fa2cu_server_open", "fa2cu_server_submit", "fa2cu_server_wait",
    "fa2cu_server_collect",
    "fa2cu_server_stats", "fa2cu_server_close", "fa2cu_layout_footprint",
    "fa2cu_graph_prep", "fa2cu_layout_open_edges", "fa2cu_full_run_edges",
)
