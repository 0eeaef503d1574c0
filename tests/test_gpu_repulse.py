"""fa2_gpu_repulse_exact / fa2_gpu_repulse_bh through the C interface against
the oracle (src/forceatlas2.c restated; pinned by tests/golden).

Tolerances (per-step force, norm-wise relative error
max_i |f_i - g_i| / max_i |g_i|, from identical positions): precision
"double" <= 1e-12 (the FP64 kernels keep the reference's operation order),
precision "single" <= 1e-4. With prevent_overlap (adjust) the single bar is
2e-3: near contact, d = sqrt(d2) - (r_i + r_j) cancels and float inputs carry
an absolute error of about one ulp of the coordinates, so the condition
number of the force grows like r / d (the reference's float construction
shows 2e-4 on these cases).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from forceatlas2_rc_gb300 import graphs as G
from forceatlas2_rc_gb300._abi import dptr

pytestmark = pytest.mark.gpu

TOL = {1: 1e-12, 0: 1e-4}
TOL_ADJUST_SINGLE = 2e-3


def tol(use_double, adjust):
    return TOL[1] if use_double else (TOL_ADJUST_SINGLE if adjust else TOL[0])


def f32(a):
    """Values the single-precision path represents exactly."""
    return None if a is None else np.asarray(a).astype(np.float32).astype(np.float64)


def _case(n, seed=42, coincident=0):
    n, a, b = G.pa_test_graph(n, seed=seed)
    rng = np.random.default_rng(3)
    size = rng.uniform(0.5, 4.0, n)
    pos = G.uniform_positions(n, -50, 50, seed=7)
    if coincident:
        pos[:coincident] = 1.0
    return n, a, b, size, pos


class Session:
    def __init__(self, lib, n, use_double, adjust, bh):
        self.lib = lib
        self.h = lib.fa2_gpu_open(0, use_double, n, adjust, bh, 1)
        assert self.h, lib.fa2_gpu_error()

    def close(self):
        self.lib.fa2_gpu_close(self.h)


@pytest.mark.parametrize("use_double", [1, 0])
@pytest.mark.parametrize("adjust", [0, 1])
def test_repulse_exact(cuda_lib, gpu, orc, use_double, adjust):
    n, a, b, size, pos = _case(400, coincident=10)
    if not use_double:
        pos, size = f32(pos), f32(size)
    m, _ = orc.mass(n, a, b)
    want = orc.repulse_exact(n, pos, m, size if adjust else None, adjust, 5.0)
    s = Session(cuda_lib, n, use_double, adjust, 0)
    x, y = pos[:, 0].copy(), pos[:, 1].copy()
    dx, dy = np.zeros(n), np.zeros(n)

    def call():
        rc = cuda_lib.fa2_gpu_repulse_exact(s.h, dptr(x), dptr(y), dptr(m),
                                            dptr(size if adjust else None),
                                            5.0, dptr(dx), dptr(dy))
        assert rc == 0, cuda_lib.fa2_gpu_error()

    call()
    got = np.stack([dx, dy], axis=1)
    err = rel_err(got, want)
    assert err <= tol(use_double, adjust), err
    if use_double:
        # same operations in the same order as the reference
        np.testing.assert_array_equal(got, want)
    call()  # the forces are added to dx, dy
    np.testing.assert_array_equal(np.stack([dx, dy], axis=1), 2 * got)
    t = np.zeros(3)
    cuda_lib.fa2_gpu_times(s.h, dptr(t))
    assert (t >= 0).all() and t.sum() > 0
    s.close()


@pytest.mark.parametrize("use_double", [1, 0])
@pytest.mark.parametrize("theta", [0.0, 0.5, 1.2])
@pytest.mark.parametrize("adjust", [0, 1])
def test_repulse_bh_quadtree(cuda_lib, gpu, orc, use_double, theta, adjust):
    n, a, b, size, pos = _case(500, coincident=25)
    if not use_double:
        pos, size = f32(pos), f32(size)
    m, _ = orc.mass(n, a, b)
    sz = size if adjust else None
    qt = orc.QuadTree(n, pos, m, sz)
    want = orc.repulse_bh(qt, pos, m, sz, adjust, 2.0, theta)
    s = Session(cuda_lib, n, use_double, adjust, 1)
    dx, dy = np.zeros(n), np.zeros(n)
    rc = cuda_lib.fa2_gpu_repulse_bh(s.h, C.byref(qt.t), 2.0, theta, dptr(dx),
                                     dptr(dy))
    assert rc == 0, cuda_lib.fa2_gpu_error()
    got = np.stack([dx, dy], axis=1)
    err = rel_err(got, want)
    assert err <= tol(use_double, adjust), err
    if use_double:
        np.testing.assert_array_equal(got, want)
    s.close()


def test_bh_matches_golden_reference_forces(cuda_lib, gpu, orc, golden):
    """Repulsion from the GPU + the oracle's gravity and attraction
    reproduce the reference's recorded per-step forces (BH, theta 1.2)."""
    g = golden
    n = int(g["cf_n"])
    a, b, w, size, pos = g["cf_from"], g["cf_to"], g["cf_w"], g["cf_size"], g["cf_pos"]
    m, _ = orc.mass(n, a, b)
    qt = orc.QuadTree(n, pos, m)
    s = Session(cuda_lib, n, 1, 0, 1)
    dx, dy = np.zeros(n), np.zeros(n)
    assert cuda_lib.fa2_gpu_repulse_bh(s.h, C.byref(qt.t), 10.0, 1.2, dptr(dx),
                                       dptr(dy)) == 0
    x, y = pos[:, 0].copy(), pos[:, 1].copy()
    orc.lib().orc_gravity(n, dptr(x), dptr(y), dptr(m), C.c_double(1.0), 0,
                          dptr(dx), dptr(dy))
    orc.lib().orc_attract(n, len(a), a.ctypes.data_as(C.POINTER(C.c_int)),
                          b.ctypes.data_as(C.POINTER(C.c_int)), dptr(w),
                          dptr(x), dptr(y), dptr(m), dptr(size), C.c_double(1.0),
                          0, 0, 0, dptr(dx), dptr(dy))
    np.testing.assert_array_equal(np.stack([dx, dy], 1), g["cf_0_1_1.2"])
    s.close()


def test_invalid_tree_is_rejected(cuda_lib, gpu, orc):
    n, a, b, size, pos = _case(200)
    m, _ = orc.mass(n, a, b)
    qt = orc.QuadTree(n, pos, m)
    r = 3 if qt.nreg > 3 else qt.nreg - 1
    qt.reg[r].skip = r  # a walk would loop forever
    s = Session(cuda_lib, n, 0, 0, 1)
    dx, dy = np.zeros(n), np.zeros(n)
    rc = cuda_lib.fa2_gpu_repulse_bh(s.h, C.byref(qt.t), 2.0, 1.2, dptr(dx),
                                     dptr(dy))
    assert rc != 0
    assert b"invalid Barnes-Hut tree" in cuda_lib.fa2_gpu_error()
    s.close()


def test_open_errors(cuda_lib, gpu):
    lib = cuda_lib
    nd = lib.fa2_gpu_ndevices()
    assert lib.fa2_gpu_open(nd, 0, 10, 0, 0, 1) is None
    assert b"there is no CUDA device" in lib.fa2_gpu_error()
    assert lib.fa2_gpu_open(0, 0, 0, 0, 0, 1) is None
    assert b"at most" in lib.fa2_gpu_error()
    lib.fa2_gpu_close(None)  # no-op, as the reference


def test_device_info(cuda_lib, gpu):
    from forceatlas2_rc_gb300 import gpu_devices
    d = gpu_devices()
    assert len(d) >= 1
    assert list(d[0]) == ["name", "vendor", "platform", "version", "type",
                          "memory_gb", "double"]
    assert d[0]["type"] == "GPU" and d[0]["double"] and d[0]["platform"] == "CUDA"
    assert "nvidia" in d[0]["vendor"].lower()
    assert d[0]["memory_gb"] > 1
