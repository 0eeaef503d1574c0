import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "fa2_golden.npz")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda_lib():
    """libfa2cuda.so, built in-tree if needed (nvcc cross-compiles without a
    GPU)."""
    from forceatlas2_rc_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    """A CUDA device is required: GPU tests fail (not skip) without one, so
    that a missing device or library is never mistaken for a pass."""
    n = cuda_lib.fa2_gpu_ndevices()
    assert n > 0, "no CUDA device: " + cuda_lib.fa2_gpu_error().decode()
    return 0


def rel_err(a, b):
    """Norm-wise relative error of per-node force vectors:
    max_i |a_i - b_i| / max_i |b_i|."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.sqrt((b ** 2).sum(axis=1)).max()
    num = np.sqrt(((a - b) ** 2).sum(axis=1)).max()
    return num / den if den > 0 else num
