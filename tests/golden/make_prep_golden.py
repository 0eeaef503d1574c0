"""Golden vectors of the graph preparation (tests/golden/prep_golden.npz),
recorded from the reference's own C_forceatlas2_large.

The package's src/forceatlas2.c (the .Call layer) is compiled from the
reference checkout and linked with a stand-in backend
(oracle/ref/ref_capture.c, make target `ref-capture`) that records the masses
and incidence lists C_forceatlas2_large hands to fa2_full_run. Cases cover
self-loops, repeated edges, isolated nodes, graphs with no incidences and
both coefficient modes. Re-run with:

    python tests/golden/make_prep_golden.py

Needs the reference checkout at /root/reference (this container only).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from forceatlas2_rc_gb300 import graphs as G  # noqa: E402

OUT = os.path.join(HERE, "prep_golden.npz")


def cases():
    rng = np.random.default_rng(11)
    n, a, b = G.pa_test_graph(60, seed=42)
    w = rng.uniform(0.2, 3.0, len(a))
    yield n, a, b, w, False
    yield n, a, b, w, True
    # a multigraph: self-loops, repeated pairs in both directions, isolated
    # nodes (the last 5 never appear)
    n = 40
    a = rng.integers(0, 35, 150)
    b = rng.integers(0, 35, 150)
    a[::7] = b[::7]
    a[100:110], b[100:110] = 3, 9
    a[110:115], b[110:115] = 9, 3
    w = rng.lognormal(0.0, 0.5, 150)
    yield n, a, b, w, False
    yield n, a, b, w, True
    # self-loops only, and no edges at all
    yield 3, np.array([0, 1, 1]), np.array([0, 1, 1]), np.array([1.0, 2.0, 0.5]), True
    yield 5, np.zeros(0, int), np.zeros(0, int), np.zeros(0), True
    # owners needing one and two 8-bit sort passes
    n, a, b = G.barabasi_albert(255, 3, seed=5)
    yield n, a, b, rng.lognormal(0.0, 0.5, len(a)), True
    n, a, b = G.barabasi_albert(300, 2, seed=6)
    yield n, a, b, rng.uniform(0.1, 5.0, len(a)), True


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s", "ref-capture",
                    "REF=" + os.environ.get("FA2_REF", "/root/reference")],
                   check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libfa2ref_capture.so"))
    lib.ref_error.restype = C.c_char_p
    P = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
    out = {}
    for k, (n, a, b, w, ob) in enumerate(cases()):
        a = np.ascontiguousarray(a, np.int32)
        b = np.ascontiguousarray(b, np.int32)
        w = np.ascontiguousarray(w, np.float64)
        m = len(a)
        pos = np.zeros(2 * n)
        size = np.ones(n)
        fixed = np.zeros(n, np.int32)
        res = np.zeros(2 * n)
        dpar = np.array([2.0, 1.0, 1.0, 1.2])
        flags = np.array([0, 0, int(ob), 0], np.int32)
        gpu = np.array([0, 0, 0], np.int32)
        rc = lib.ref_C_forceatlas2_large(n, m, P(a), P(b), P(w), P(pos), P(size),
                                         P(fixed), 1, P(dpar), P(flags), P(gpu),
                                         P(res))
        assert rc == 0, lib.ref_error()
        nn, ninc = C.c_int(), C.c_int()
        lib.capture_get(C.byref(nn), C.byref(ninc), None, None, None, None)
        mass = np.zeros(n)
        off = np.zeros(n + 1, np.int32)
        node = np.zeros(max(ninc.value, 1), np.int32)
        coef = np.zeros(max(ninc.value, 1))
        lib.capture_get(C.byref(nn), C.byref(ninc), P(mass), P(off), P(node), P(coef))
        out.update({f"prep_{k}_n": n, f"prep_{k}_from": a, f"prep_{k}_to": b,
                    f"prep_{k}_w": w, f"prep_{k}_outbound": int(ob),
                    f"prep_{k}_mass": mass, f"prep_{k}_off": off,
                    f"prep_{k}_node": node[:ninc.value],
                    f"prep_{k}_coef": coef[:ninc.value]})
        print(f"case {k}: n={n} m={m} incidences={ninc.value}")
    out["ncases"] = k + 1
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
