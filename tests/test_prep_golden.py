"""The graph preparation of C_forceatlas2_large (masses, symmetric incidence
lists, coefficients) against golden vectors recorded from the reference's
own code (tests/golden/make_prep_golden.py): the oracle's restatement and
the host Graph() bit for bit (CPU), and the device preparation
(fa2cu_graph_prep) bit for bit (GPU)."""
import os

import numpy as np
import pytest

from conftest import ROOT

PREP = os.path.join(ROOT, "tests", "golden", "prep_golden.npz")


@pytest.fixture(scope="module")
def prep():
    return np.load(PREP)


def cases(prep):
    for k in range(int(prep["ncases"])):
        g = {x: prep[f"prep_{k}_{x}"] for x in ("n", "from", "to", "w", "outbound",
                                                "mass", "off", "node", "coef")}
        g["n"] = int(g["n"])
        g["outbound"] = bool(g["outbound"])
        yield k, g


def check(k, g, mass, off, node, coef):
    ninc = int(g["off"][-1])
    np.testing.assert_array_equal(mass, g["mass"], err_msg=f"case {k} mass")
    np.testing.assert_array_equal(off, g["off"], err_msg=f"case {k} inc_off")
    np.testing.assert_array_equal(node[:ninc], g["node"], err_msg=f"case {k} inc_node")
    np.testing.assert_array_equal(coef[:ninc], g["coef"], err_msg=f"case {k} inc_coef")


def test_oracle_prepare_large_golden(prep, orc):
    for k, g in cases(prep):
        r = orc.prepare_large(g["n"], g["from"], g["to"], g["w"], outbound=g["outbound"])
        check(k, g, r.mass, r.inc_off, r.inc_node, r.inc_coef)


def test_host_graph_golden(prep):
    from forceatlas2_rc_gb300.layout import Graph
    for k, g in cases(prep):
        r = Graph(g["n"], g["from"], g["to"], g["w"], outbound=g["outbound"])
        check(k, g, r.mass, r.inc_off, r.inc_node, r.inc_coef)


@pytest.mark.gpu
def test_device_prep_golden(prep, gpu):
    from forceatlas2_rc_gb300.layout import prepare_graph_device
    for k, g in cases(prep):
        r = prepare_graph_device(g["n"], g["from"], g["to"], g["w"],
                                 dissuade_hubs=g["outbound"])
        check(k, g, r.mass, r.inc_off, r.inc_node, r.inc_coef)
