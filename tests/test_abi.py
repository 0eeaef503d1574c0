"""The C interface of libfa2cuda.so, without a GPU: it builds, loads, exports
every entry point that include/*.h declares, and fails cleanly (status and
message, no crash) when no device is present. Also checks that the
package's own src/forceatlas2.c links against it as a drop-in (where the
reference checkout is present)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in ("fa2.h", "fa2_cuda.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(fa2(?:cu)?_[a-z_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_exports_every_declared_entry_point(cuda_lib):
    from forceatlas2_rc_gb300 import _lib
    declared = declared_functions()
    # defined by the package's forceatlas2.c, not by the backend
    declared.discard("fa2_update_speed")
    assert declared, "no declaration found"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    missing = declared - exported
    assert not missing, f"not exported: {sorted(missing)}"
    assert declared <= set(_lib.EXPORTED) | {"fa2_gpu_error"}
    # nothing that would clash with the package's own symbols
    assert "fa2_update_speed" not in exported


def test_no_device_fails_cleanly(cuda_lib):
    lib = cuda_lib
    if lib.fa2_gpu_ndevices() > 0:
        pytest.skip("a GPU is present")
    assert lib.fa2_gpu_ndevices() == 0
    assert b"no CUDA device" in lib.fa2_gpu_error()
    assert lib.fa2_gpu_open(0, 0, 10, 0, 0, 1) is None
    assert lib.fa2_now() > 0


def test_open_rejects_bad_sizes(cuda_lib):
    """Argument checks happen before any device work."""
    from forceatlas2_rc_gb300._abi import FullParams
    lib = cuda_lib
    p = FullParams()
    p.n = 1
    pos = np.zeros(2)
    t = np.zeros(7)
    rc = lib.fa2_full_run(C.byref(p), pos.ctypes.data_as(C.POINTER(C.c_double)),
                          t.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc != 0
    assert b"between 2 and 67 million" in lib.fa2_gpu_error()


def test_invalid_csr_is_rejected(cuda_lib):
    from forceatlas2_rc_gb300._abi import FullParams, dptr, iptr
    lib = cuda_lib
    n = 4
    off = np.array([0, 1, 2, 3, 4], np.int32)
    node = np.array([1, 0, 3, 7], np.int32)  # 7 does not exist
    coef = np.ones(4)
    mass = np.ones(n)
    p = FullParams()
    p.n = n
    p.inc_off, p.inc_node, p.inc_coef, p.mass = iptr(off), iptr(node), dptr(coef), dptr(mass)
    p.iterations = 1
    pos = np.zeros(2 * n)
    assert lib.fa2cu_layout_open(C.byref(p), dptr(pos), 0) is None
    assert b"does not exist" in lib.fa2_gpu_error()


def test_reference_driver_links_against_backend(cuda_lib):
    """src/forceatlas2.c (the .Call layer) + libfa2cuda.so instead of the
    OpenCL backend: the link resolves every symbol and C_forceatlas2_large
    reaches fa2_full_run."""
    import oracle
    if oracle.REF_SRC and os.path.isdir(os.path.join(oracle.REF_SRC, "src")):
        subprocess.run(["make", "-C", oracle.HERE, "-s", "ref-cuda",
                        f"REF={oracle.REF_SRC}"], check=True)
    if not os.path.exists(oracle.REF_CUDA_LIB):
        pytest.skip("the reference's .Call layer was not built (no checkout)")
    lib = C.CDLL(oracle.REF_CUDA_LIB)
    lib.ref_error.restype = C.c_char_p
    n = 10
    frm = np.arange(9, dtype=np.int32)
    to = frm + 1
    w = np.ones(9)
    pos = np.random.default_rng(0).random(20)
    size = np.ones(n)
    fixed = np.zeros(n, np.int32)
    out = np.zeros(20)
    dpar = np.array([2.0, 1.0, 1.0, 1.2])
    fl = np.zeros(4, np.int32)
    gpu = np.array([0, 0, 0], np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    rc = lib.ref_C_forceatlas2_large(n, 9, P(frm), P(to), P(w), P(pos), P(size),
                                     P(fixed), 5, P(dpar), P(fl), P(gpu), P(out))
    if cuda_lib.fa2_gpu_ndevices() == 0:
        assert rc == 1
        assert b"CUDA device" in lib.ref_error()
    else:
        assert rc == 0
        assert np.isfinite(out).all()
