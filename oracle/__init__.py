"""ORACLE -- test infrastructure only.

Python access to the CPU restatement of the ForceAtlas2 step
(oracle/_build/libfa2oracle.so, built from fa2_oracle.c) and, where it was
built, to the package's own C code compiled from the reference checkout
(oracle/_ref/libfa2ref.so). Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module; the product never
does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

from forceatlas2_rc_gb300._abi import FullParams, Tree, Region, Node, dptr, iptr, uptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfa2oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfa2ref.so")
REF_CUDA_LIB = os.path.join(HERE, "_ref", "libfa2ref_cuda.so")
# the reference checkout, where one is present: FA2_REF in the environment
# or the ref_src given to build() (no default: the GPU host has none)
REF_SRC = os.environ.get("FA2_REF", "")


def build(ref: bool = False, quiet: bool = True, ref_src: str = "") -> None:
    """Compile the oracle, and when asked and the reference's sources are
    at ref_src (or FA2_REF) the reference harness (oracle/_ref/libfa2ref.so)
    and, if libfa2cuda.so is built, the reference's .Call layer linked
    against it (libfa2ref_cuda.so), with oracle/Makefile."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "-s"], check=True, stdout=out)
    src = ref_src or REF_SRC
    if ref and src and os.path.isdir(os.path.join(src, "src")):
        subprocess.run(["make", "-C", HERE, "-s", "ref", f"REF={src}"], check=True,
                       stdout=out)
        cuda = os.path.join(os.path.dirname(HERE), "forceatlas2_rc_gb300", "libfa2cuda.so")
        if os.path.exists(cuda):
            subprocess.run(["make", "-C", HERE, "-s", "ref-cuda", f"REF={src}"], check=True,
                           stdout=out)


class OrcOpts(C.Structure):
    _fields_ = [("scaling", C.c_double), ("gravity", C.c_double),
                ("jitter_tolerance", C.c_double), ("theta", C.c_double),
                ("strong", C.c_int), ("linlog", C.c_int),
                ("outbound", C.c_int), ("adjust", C.c_int),
                ("barnes_hut", C.c_int), ("threads", C.c_int)]


@dataclass
class Opts:
    """Settings of C_forceatlas2 (dpar and flags)."""
    scaling: float = 2.0
    gravity: float = 1.0
    jitter_tolerance: float = 1.0
    theta: float = 1.2
    strong: bool = False
    linlog: bool = False
    outbound: bool = False
    adjust: bool = False
    barnes_hut: bool = False
    threads: int = 1

    def c(self) -> OrcOpts:
        return OrcOpts(self.scaling, self.gravity, self.jitter_tolerance,
                       self.theta, int(self.strong), int(self.linlog),
                       int(self.outbound), int(self.adjust),
                       int(self.barnes_hut), int(self.threads))

    def dpar(self):
        return np.array([self.scaling, self.gravity, self.jitter_tolerance,
                         self.theta], dtype=np.float64)

    def flags5(self):
        return np.array([self.strong, self.linlog, self.outbound, self.adjust,
                         self.barnes_hut], dtype=np.int32)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        _lib.orc_forces.restype = C.c_int
        _lib.orc_layout.restype = C.c_int
        _lib.orc_layout_trace.restype = C.c_int
        _lib.orc_prepare_large.restype = C.c_int
        for s in ("f", "d"):
            getattr(_lib, f"orc_pipe_forces_{s}").restype = C.c_int
            getattr(_lib, f"orc_pipe_run_{s}").restype = C.c_int
        _lib.orc_pipe_forces_m.restype = C.c_int
    return _lib


def ref_lib():
    """The reference's own C code, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        _ref = C.CDLL(REF_LIB)
        _ref.ref_error.restype = C.c_char_p
        _ref.ref_tree.restype = C.c_int
    return _ref


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _pos_cols(pos):
    """(n, 2) positions -> x then y, as the package passes them."""
    pos = np.asarray(pos, dtype=np.float64)
    return np.ascontiguousarray(pos.T.reshape(-1))


# ---- Part 1: src/forceatlas2.c ---------------------------------------------

def mass(n, frm, to):
    out = np.empty(n, np.float64)
    mean = C.c_double()
    frm, to = _i32(frm), _i32(to)
    lib().orc_mass(n, len(frm), iptr(frm), iptr(to), dptr(out), C.byref(mean))
    return out, mean.value


def forces(n, frm, to, w, pos, size, opts: Opts, which="oracle"):
    """Forces of one iteration at `pos` ((n, 2)), as an (n, 2) array."""
    frm, to, w = _i32(frm), _i32(to), _f64(w)
    xy = _pos_cols(pos)
    size = _f64(size if size is not None else np.ones(n))
    f = np.zeros(2 * n, np.float64)
    if which == "oracle":
        o = opts.c()
        rc = lib().orc_forces(n, len(frm), iptr(frm), iptr(to), dptr(w),
                              dptr(xy), dptr(size), C.byref(o), dptr(f))
    else:
        rc = ref_lib().ref_forces(n, len(frm), iptr(frm), iptr(to), dptr(w),
                                  dptr(xy), dptr(size), dptr(opts.dpar()),
                                  iptr(opts.flags5()), dptr(f))
    if rc:
        raise RuntimeError("oracle forces failed")
    return f.reshape(2, n).T.copy()


def layout(n, frm, to, w, pos, size, fixed, iterations, opts: Opts,
           which="oracle"):
    """C_forceatlas2 on the CPU: the layout after `iterations`."""
    frm, to, w = _i32(frm), _i32(to), _f64(w)
    xy = _pos_cols(pos)
    size = _f64(size if size is not None else np.ones(n))
    fixed = _i32(fixed if fixed is not None else np.zeros(n))
    if which == "oracle":
        o = opts.c()
        rc = lib().orc_layout(n, len(frm), iptr(frm), iptr(to), dptr(w),
                              dptr(xy), dptr(size), iptr(fixed), iterations,
                              C.byref(o))
        if rc:
            raise RuntimeError("oracle layout failed")
        return xy.reshape(2, n).T.copy()
    out = np.zeros(2 * n, np.float64)
    rc = ref_lib().ref_C_forceatlas2(
        n, len(frm), iptr(frm), iptr(to), dptr(w), dptr(xy), dptr(size),
        iptr(fixed), iterations, dptr(opts.dpar()), iptr(opts.flags5()),
        opts.threads, dptr(out), dptr(None))
    if rc:
        raise RuntimeError(ref_lib().ref_error().decode())
    return out.reshape(2, n).T.copy()


def layout_trace(n, frm, to, w, pos, size, fixed, iterations, opts: Opts):
    """Positions before the first iteration and after each one, as an
    (iterations + 1, n, 2) array."""
    frm, to, w = _i32(frm), _i32(to), _f64(w)
    xy = _pos_cols(pos)
    size = _f64(size if size is not None else np.ones(n))
    fixed = _i32(fixed if fixed is not None else np.zeros(n))
    tr = np.zeros((iterations + 1) * 2 * n)
    o = opts.c()
    rc = lib().orc_layout_trace(n, len(frm), iptr(frm), iptr(to), dptr(w),
                                dptr(xy), dptr(size), iptr(fixed), iterations,
                                C.byref(o), dptr(tr))
    if rc:
        raise RuntimeError("oracle layout failed")
    return tr.reshape(iterations + 1, 2, n).transpose(0, 2, 1).copy()


class QuadTree:
    """A Gephi quadtree built by the oracle, in fa2_tree layout (the input of
    fa2_gpu_repulse_bh). Keeps its arrays alive."""

    def __init__(self, n, pos, mass_, size=None, threads=1):
        self.n = n
        xy = _pos_cols(pos)
        self._x, self._y = xy[:n].copy(), xy[n:].copy()
        self._m = _f64(mass_)
        self._s = _f64(size) if size is not None else None
        self.reg = (Region * (2 * n))()
        self.perm = np.zeros(n, np.int32)
        self.cnt = np.zeros(4 * n, np.int32)
        self.buf0 = (Node * n)()
        self.buf1 = (Node * n)()
        self.px = np.zeros(n)
        self.py = np.zeros(n)
        self.pm = np.zeros(n)
        self.ps = np.zeros(n) if size is not None else None
        t = Tree()
        t.reg = C.cast(self.reg, C.POINTER(Region))
        t.perm = iptr(self.perm)
        t.cnt = iptr(self.cnt)
        t.buf[0] = C.cast(self.buf0, C.POINTER(Node))
        t.buf[1] = C.cast(self.buf1, C.POINTER(Node))
        t.px, t.py, t.pm = dptr(self.px), dptr(self.py), dptr(self.pm)
        t.ps = dptr(self.ps)
        self.t = t
        lib().orc_tree_build_mt(C.byref(t), n, dptr(self._x), dptr(self._y),
                                dptr(self._m), dptr(self._s), int(threads))

    @property
    def nreg(self):
        return self.t.nreg

    def regions(self):
        """(nreg, 10) array: mass, cx, cy, size, start, count, child, nchild,
        skip, buf."""
        out = np.zeros((self.nreg, 10))
        for r in range(self.nreg):
            g = self.reg[r]
            out[r] = (g.mass, g.cx, g.cy, g.size, g.start, g.count, g.child,
                      g.nchild, g.skip, g.buf)
        return out


def ref_tree(n, pos, mass_):
    """The reference's own tree_build: (regions (nreg, 10), perm, pxyz)."""
    xy = _pos_cols(pos)
    regs = np.zeros((2 * n, 10))
    perm = np.zeros(n, np.int32)
    pxyz = np.zeros(3 * n)
    nreg = ref_lib().ref_tree(n, dptr(xy), dptr(_f64(mass_)), dptr(regs),
                              iptr(perm), dptr(pxyz))
    return regs[:nreg], perm, pxyz


def repulse_bh(qt: QuadTree, pos, mass_, size, adjust, scaling, theta,
               threads=1):
    n = qt.n
    xy = _pos_cols(pos)
    f = np.zeros(2 * n)
    lib().orc_repulse_bh(n, C.byref(qt.t), dptr(xy[:n].copy()),
                         dptr(xy[n:].copy()), dptr(_f64(mass_)),
                         dptr(_f64(size) if size is not None else None),
                         int(adjust), C.c_double(scaling), C.c_double(theta),
                         threads, dptr(f[:n]), dptr(f[n:]))
    return f.reshape(2, n).T.copy()


def repulse_exact(n, pos, mass_, size, adjust, scaling, threads=1):
    xy = _pos_cols(pos)
    f = np.zeros(2 * n)
    x, y = xy[:n].copy(), xy[n:].copy()
    fx, fy = np.zeros(n), np.zeros(n)
    lib().orc_repulse_exact(n, dptr(x), dptr(y), dptr(_f64(mass_)),
                            dptr(_f64(size) if size is not None else None),
                            int(adjust), C.c_double(scaling), threads,
                            dptr(fx), dptr(fy))
    return np.stack([fx, fy], axis=1)


def update_speed(n, sw, tr, jt, speed, eff, which="oracle"):
    s, e = C.c_double(speed), C.c_double(eff)
    fn = lib().orc_update_speed if which == "oracle" else ref_lib().ref_update_speed
    fn(n, C.c_double(sw), C.c_double(tr), C.c_double(jt), C.byref(s),
       C.byref(e))
    return s.value, e.value


# ---- the symmetric CSR of C_forceatlas2_large --------------------------------

@dataclass
class LargeGraph:
    """Inputs of fa2_full_run prepared as C_forceatlas2_large does."""
    n: int
    mass: np.ndarray
    inc_off: np.ndarray
    inc_node: np.ndarray
    inc_coef: np.ndarray


def prepare_large(n, frm, to, w, outbound=False) -> LargeGraph:
    frm, to, w = _i32(frm), _i32(to), _f64(w)
    m = len(frm)
    mass_ = np.zeros(n)
    off = np.zeros(n + 1, np.int32)
    node = np.zeros(max(2 * m, 1), np.int32)
    coef = np.zeros(max(2 * m, 1))
    ninc = lib().orc_prepare_large(n, m, iptr(frm), iptr(to), dptr(w),
                                   int(outbound), dptr(mass_), iptr(off),
                                   iptr(node), dptr(coef))
    return LargeGraph(n, mass_, off, node[:max(ninc, 1)].copy(),
                      coef[:max(ninc, 1)].copy())


def full_params(g: LargeGraph, size=None, fixed=None, scaling=2.0,
                gravity=1.0, theta=1.2, jitter_tolerance=1.0, strong=False,
                linlog=False, adjust=False, iterations=1, use_double=False):
    """A FullParams over `g`; the returned tuple keeps the arrays alive."""
    n = g.n
    size = _f64(size if size is not None else np.ones(n))
    fixed = _i32(fixed if fixed is not None else np.zeros(n))
    p = FullParams()
    p.n = n
    p.inc_off, p.inc_node = iptr(g.inc_off), iptr(g.inc_node)
    p.inc_coef, p.mass = dptr(g.inc_coef), dptr(g.mass)
    p.size, p.fixed = dptr(size), iptr(fixed)
    p.any_fixed = int(fixed.any())
    p.scaling, p.gravity, p.theta = scaling, gravity, theta
    p.jitter_tolerance = jitter_tolerance
    p.strong, p.linlog, p.adjust = int(strong), int(linlog), int(adjust)
    p.iterations = iterations
    p.device, p.use_double, p.profile = 0, int(use_double), 0
    return p, (size, fixed, g)


# ---- Part 2: inst/opencl/pipeline.cl ----------------------------------------

def pipe_build(n, pos, mass_, precision="f", which="oracle"):
    """Keys, order, child, range, parent and ni of the Karras construction."""
    xy = _pos_cols(pos)
    key = np.zeros(n, np.uint32)
    order = np.zeros(n, np.uint32)
    child = np.zeros(2 * (n - 1), np.int32)
    rng = np.zeros(2 * (n - 1), np.int32)
    parent = np.zeros(2 * n - 1, np.int32)
    ni = np.zeros(4 * (n - 1))
    if which == "oracle":
        fn = getattr(lib(), f"orc_pipe_build_{precision}")
    else:
        fn = getattr(ref_lib(), f"ref_pipe_build_{precision}")
    fn(n, dptr(xy), dptr(_f64(mass_)), uptr(key), uptr(order), iptr(child),
       iptr(rng), iptr(parent), dptr(ni))
    return dict(key=key, order=order, child=child, range=rng, parent=parent,
                ni=ni.reshape(-1, 4) if n > 1 else ni)


def pipe_forces(p: FullParams, pos, precision="f", which="oracle"):
    """precision "f" / "d": the reference's float / double construction;
    "m": the FP32 path of libfa2cuda.so (double construction over the
    float-rounded inputs, float walk and attraction)."""
    n = p.n
    xy = _pos_cols(pos)
    f = np.zeros(2 * n)
    if which == "oracle":
        fn = getattr(lib(), f"orc_pipe_forces_{precision}")
    else:
        fn = getattr(ref_lib(), f"ref_pipe_forces_{precision}")
    rc = fn(C.byref(p), dptr(xy), dptr(f))
    if rc:
        raise RuntimeError("pipeline forces failed")
    return f.reshape(2, n).T.copy()


def pipe_run(p: FullParams, pos, precision="f", totals_fp64=True,
             which="oracle"):
    n = p.n
    xy = _pos_cols(pos)
    if which == "oracle":
        rc = getattr(lib(), f"orc_pipe_run_{precision}")(C.byref(p), dptr(xy),
                                                         int(totals_fp64))
    else:
        rc = getattr(ref_lib(), f"ref_pipe_run_{precision}")(C.byref(p),
                                                             dptr(xy))
    if rc:
        raise RuntimeError(f"pipeline run failed ({rc})")
    return xy.reshape(2, n).T.copy()
