"""The oracle's restatement of the single-precision path ("m": the double
construction over float-rounded inputs, the float walk with its node pairs
deferred, gravity and attraction summed apart from the repulsion and added
to it, the hubs' attraction as a warp's sum) against the oracle's double
pipeline ("d", pipeline.cl in double) on the CPU: within the FP32 bar of
1e-4 (norm-wise, per step, from identical positions), reproducible, and not
the double result itself. The GPU tests hold the device's FP32 path to this
restatement within 1e-5."""
import numpy as np
import pytest

from conftest import rel_err
from forceatlas2_rc_gb300 import graphs as G


def f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


CASES = [
    # a Barabasi-Albert graph with a hub of 300 incidences (warp-summed
    # attraction, compensated walk sums), lognormal weights
    ("ba_hub", dict(theta=1.2)),
    # linlog with dissuade_hubs (outbound coefficients)
    ("ba_linlog_outbound", dict(theta=1.2, linlog=True)),
    # prevent_overlap, node sizes in [0.5, 3]
    ("ba_adjust", dict(theta=1.2, adjust=True)),
    # an opening angle that opens more regions
    ("ba_theta05", dict(theta=0.5)),
]


@pytest.mark.parametrize("name,opts", CASES)
def test_fp32_restatement_within_the_fp32_bar(orc, name, opts):
    n, a, b = G.barabasi_albert(3000, 3, seed=41)
    rng = np.random.default_rng(42)
    if name == "ba_hub":
        a = np.concatenate([a, np.zeros(300, np.int32)])
        b = np.concatenate([b, rng.choice(np.arange(1, n), 300, replace=False)
                            .astype(np.int32)])
    w = rng.lognormal(0.0, 0.5, len(a))
    pos = f32(G.uniform_positions(n, 0.0, 1000.0, seed=43))
    size = f32(rng.uniform(0.5, 3.0, n)) if opts.get("adjust") else None
    go = orc.prepare_large(n, a, b, w, outbound=name.endswith("outbound"))
    p, keep = orc.full_params(go, size=size, scaling=2.0, gravity=1.0, **opts)
    fm = orc.pipe_forces(p, pos, "m")
    fd = orc.pipe_forces(p, pos, "d")
    # prevent_overlap's near-contact force is ill-conditioned in float
    tol = 2e-3 if opts.get("adjust") else 1e-4
    assert rel_err(fm, fd) <= tol, name
    assert not np.array_equal(fm, fd), name
    np.testing.assert_array_equal(orc.pipe_forces(p, pos, "m"), fm)
