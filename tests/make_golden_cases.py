"""Small deterministic oracle cases whose outputs are committed as golden
vectors (tests/golden/oracle_golden.npz) by tests/golden/make_golden.py.

Inputs are built from seeded generators only, so the GPU machine reproduces them
without the reference tree.
"""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _params(name):
    with open(os.path.join(GOLDEN, "params_%s.json" % name)) as fh:
        return json.load(fh)


def case_lvelva():
    rng = np.random.default_rng(11)
    n, dx = 32, 50e3
    w = rng.standard_normal((n, n)) * 50
    cf = rng.standard_normal((n, n)) * 1e5
    mask = (rng.random((n, n)) > 0.1).astype(np.uint8)
    D = 1e24 * (1 + rng.random((n, n)))
    eta = 1e21 * (1 + rng.random((n, n)))
    R = 1 + 0.2 * rng.random((n, n))
    kap = O.kappa(n, n, dx, dx)
    dxm = np.full((n, n), dx)
    return {"dwdt": O.lvelva(w, cf, mask, 9.81, 0.28, D, eta, R, kap, dxm, dxm, 31557600.0)}


def case_conv():
    rng = np.random.default_rng(12)
    n, dx = 24, 50e3
    M = 2 * n - 1
    GE = O.elastic_green(n, n, dx)
    GN = O.zss_green(n, n, 5.972e24, 6.378e6, dx)
    x = rng.standard_normal((n, n)) * 1e7
    return {"GE": GE, "GN": GN, "we": O.conv(O.kernel_spectrum(GE, M), x, M),
            "dz": O.conv(O.kernel_spectrum(GN, M), x, M)}


def _run(p, n, dx, H, z, nsteps, dtt=10.0):
    m = O.Model(p, n, n, dx, dx)
    b = O.make_bsl()
    m.init_state(z, np.zeros_like(H), 0.0, b)
    for k in range(1, nsteps + 1):
        assert m.update(H, k * dtt, b) == 0
    out = {k: m.field(k) for k in ("w", "we", "z_bed", "dz_ss", "dwdt", "canom_full")}
    s = m.scalars()
    out["clock"] = np.array([s["t"], s["dt"], s["n_accept"], s["n_reject"]])
    m.close()
    return out


def _disc(n, dx, r0=1000e3, h0=1000.0):
    xc = (np.arange(n) - (n - 1) / 2.0) * dx
    return np.where(xc[None, :] ** 2 + xc[:, None] ** 2 <= r0 ** 2, h0, 0.0)


def case_test1d():
    p = _params("test1d")
    n, dx = 31, 200e3
    return _run(p, n, dx, _disc(n, dx), np.full((n, n), 1e6), 20)


def case_test2c():
    p = _params("test2c")
    n, dx = 31, 200e3
    return _run(p, n, dx, _disc(n, dx), np.full((n, n), 1e6), 10)


def case_test3a():
    p = _params("test3a")
    n, dx = 31, 200e3
    return _run(p, n, dx, _disc(n, dx), np.full((n, n), 1e6), 10)


CASES = {"lvelva": case_lvelva, "conv": case_conv, "test1d": case_test1d, "test2c": case_test2c,
         "test3a": case_test3a}
