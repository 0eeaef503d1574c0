"""ctypes mirrors of the C structures declared in include/fa2.h.

Only layouts live here (no library is loaded), so that both the package and
its tests can describe the C interface without a GPU.
"""
from __future__ import annotations

import ctypes as C

INTERRUPT_FN = C.CFUNCTYPE(C.c_int)


class Region(C.Structure):
    """fa2_region (reference src/fa2.h:21-27)."""
    _fields_ = [("mass", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
                ("size", C.c_double), ("start", C.c_int), ("count", C.c_int),
                ("child", C.c_int), ("nchild", C.c_int), ("skip", C.c_int),
                ("buf", C.c_int)]


class Node(C.Structure):
    """fa2_node (reference src/fa2.h:30-33)."""
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("m", C.c_double),
                ("idx", C.c_int)]


class Tree(C.Structure):
    """fa2_tree (reference src/fa2.h:35-44)."""
    _fields_ = [("reg", C.POINTER(Region)), ("nreg", C.c_int),
                ("perm", C.POINTER(C.c_int)), ("cnt", C.POINTER(C.c_int)),
                ("buf", C.POINTER(Node) * 2),
                ("px", C.POINTER(C.c_double)), ("py", C.POINTER(C.c_double)),
                ("pm", C.POINTER(C.c_double)), ("ps", C.POINTER(C.c_double))]


class DevInfo(C.Structure):
    """fa2_gpu_devinfo (reference src/fa2.h:50-58)."""
    _fields_ = [("name", C.c_char * 128), ("vendor", C.c_char * 128),
                ("platform", C.c_char * 128), ("version", C.c_char * 128),
                ("is_gpu", C.c_int), ("has_double", C.c_int),
                ("memory", C.c_double)]


class FullParams(C.Structure):
    """fa2_full_params (reference src/fa2.h:97-115)."""
    _fields_ = [("n", C.c_int),
                ("inc_off", C.POINTER(C.c_int)),
                ("inc_node", C.POINTER(C.c_int)),
                ("inc_coef", C.POINTER(C.c_double)),
                ("mass", C.POINTER(C.c_double)),
                ("size", C.POINTER(C.c_double)),
                ("fixed", C.POINTER(C.c_int)),
                ("any_fixed", C.c_int),
                ("scaling", C.c_double), ("gravity", C.c_double),
                ("theta", C.c_double), ("jitter_tolerance", C.c_double),
                ("strong", C.c_int), ("linlog", C.c_int), ("adjust", C.c_int),
                ("iterations", C.c_int),
                ("device", C.c_int), ("use_double", C.c_int),
                ("profile", C.c_int),
                ("source", C.c_char_p),
                ("interrupted", INTERRUPT_FN)]


FA2_FULL_NTIMES = 7
FULL_TIME_NAMES = ("total", "codes", "sort", "tree", "repulsion",
                   "attraction", "move")


class ServerConfig(C.Structure):
    """fa2cu_server_config (include/fa2_cuda.h)."""
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_double),
                ("max_jobs", C.c_int), ("chunk", C.c_int), ("policy", C.c_int)]


def dptr(a):
    """double* of a contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return C.POINTER(C.c_double)()
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    """int* of a contiguous int32 numpy array (or NULL for None)."""
    if a is None:
        return C.POINTER(C.c_int)()
    return a.ctypes.data_as(C.POINTER(C.c_int))


def uptr(a):
    """uint32_t* of a contiguous uint32 numpy array."""
    return a.ctypes.data_as(C.POINTER(C.c_uint32))
