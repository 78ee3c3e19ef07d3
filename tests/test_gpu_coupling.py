"""Barystatic sea-level coupling, step-control safety and the reference-API
mirror, GPU (through the C ABI) against the oracle.

* bsl methods file, fastiso and mixed, with a constant ocean surface and with
  an A_ocean(bsl) table (interp_0d): bsl_now, deltaV_bsl and dbsl_total
  within 1e-10, masks bit-exact, every update of a ramped ice load
  (src/fastisostasy.f90:766-775, src/barysealevel.f90:195-252).
* dt_min floor and the per-update rejection limit: the GPU and the oracle
  fail at the same update with FI_E_STEP after the same attempts.
* LLRA with a load that reaches the domain corners (relaxation rates carry
  no corner correction, src/fastisostasy.f90:693-714).
* isos_init from a namelist file -> isos_init_state -> bsl_update +
  isos_update every dtt -> isos%out, the reference driver's loop
  (tests/test_isostasy.f90:362-372), against the oracle.
"""
import os

import numpy as np
import pytest

from fastisostasy_gb300 import _lib
from fastisostasy_gb300 import isostasy as I
from fastisostasy_gb300 import params as P
from fastisostasy_gb300 import workloads as W
from fastisostasy_gb300.isostasy import Domain
from harness import gpu_bsl, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL64 = 1e-10
MASKS = ["maskocean", "maskgrounded", "maskcontinent"]

# sea-level series (time [yr], bsl [m]) and the ocean-area table (bsl [m],
# A_ocean [m^2]) that replace the reference's file readers
SERIES = (np.array([-500.0, 0.0, 40.0, 90.0, 400.0]), np.array([-3.0, 0.0, -12.0, 5.0, 8.0]))
AOCEAN = (np.array([-130.0, -60.0, -10.0, 0.0, 20.0]), np.array([3.30e14, 3.45e14, 3.58e14, 3.625e14, 3.70e14]))


def make_bsl_pair(method, constant_ocean):
    """The same bsl_class for the GPU (fi_bsl) and the oracle (orc_bsl)."""
    import ctypes as C
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in SERIES + AOCEAN]
    dp = C.POINTER(C.c_double)
    pairs = []
    for b in (gpu_bsl(method), O.make_bsl(method)):
        b.constant_ocean_surface = constant_ocean
        b.series_t, b.series_v = keep[0].ctypes.data_as(dp), keep[1].ctypes.data_as(dp)
        b.n_series = len(keep[0])
        b.bsl_vec, b.aocean_vec = keep[2].ctypes.data_as(dp), keep[3].ctypes.data_as(dp)
        b.n_aocean = len(keep[2])
        pairs.append(b)
    return pairs[0], pairs[1], keep


@pytest.mark.parametrize("method,constant_ocean", [(1, 1), (2, 1), (2, 0), (3, 0), (3, 1)])
def test_barystatic_coupling(method, constant_ocean):
    """Interactive sea level on a rectangular domain with a ramped ice load
    (so that the ice volume above flotation changes every update)."""
    wl = W.config3(nx_ice=40, ny_ice=72, dx=20e3, nx_pad=64, ny_pad=96)
    wl.switch_on = 95.0
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=0)
    orc = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
    bg, bo, keep = make_bsl_pair(method, constant_ocean)
    L = _lib.load()
    L.fi_bsl_update(bg, 0.0)
    O.lib().orc_bsl_update(bo, 0.0)
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)
    assert orc.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bo) == 0
    moved = 0
    for k in range(1, 11):
        t = 10.0 * k
        L.fi_bsl_update(bg, t)
        O.lib().orc_bsl_update(bo, t)
        assert abs(bg.A_ocean_now - bo.A_ocean_now) <= 1e-12 * bo.A_ocean_now
        dom.update(wl.H_at(t), t, bg)
        assert orc.update(wl.H_at(t), t, bo) == 0
        sg, so = dom.scalars(), orc.scalars()
        assert abs(bg.bsl_now - bo.bsl_now) <= TOL64 * max(1.0, abs(bo.bsl_now)), (k, bg.bsl_now, bo.bsl_now)
        for key in ("V_af", "V_den"):
            assert abs(sg[key] - so[key]) <= 1e-12 * max(1.0, abs(so[key])), (k, key)
        scale = max(abs(so["V_af"]), abs(so["V_den"]), 1.0) * 1e-12
        for key in ("deltaV_bsl", "dbsl_total"):
            # a difference of two volume sums: its rounding is that of the sums
            assert abs(sg[key] - so[key]) <= scale + TOL64 * abs(so[key]), (k, key, sg[key], so[key])
        for m in MASKS:
            assert np.array_equal(dom.field(m), orc.field(m)), (k, m)
        for f in ("w", "z_ss", "z_bed", "we"):
            b = orc.field(f)
            assert rel(dom.field(f), b) <= TOL64 or np.abs(b).max() == 0, (k, f)
        moved += so["deltaV_bsl"] != 0.0
    assert moved >= 5
    if method in (2, 3):
        assert bo.bsl_now != 0.0
    dom.close()
    orc.close()
    del keep


def _stiff(dt_min=1e-10):
    """A disc experiment whose tolerance forces rejections."""
    p = dict(P.DEFAULTS)
    p.update(atol=1e-9, rtol=1e-12, dt_min=dt_min, stage_mode=0)
    n, dx = 31, 200e3
    return W.Workload(name="stiff", params=p, nx_ice=n, ny_ice=n, dx=dx, z_bed=np.full((n, n), 1e6),
                      H_final=W.disc(n, n, dx))


def _run_until_failure(wl, max_rej, precision, updates=6):
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
    if max_rej:
        assert dom.L.fi_set_max_rejections(dom.h, max_rej) == 0
    b = gpu_bsl()
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
    for k in range(1, updates + 1):
        try:
            dom.update(wl.H_final, 10.0 * k, b)
        except _lib.FiError as e:
            sc = dom.scalars()
            dom.close()
            return e.code, k, sc
    sc = dom.scalars()
    dom.close()
    return 0, updates, sc


def _oracle_until_failure(wl, max_rej, updates=6):
    O.set_max_rejections(max_rej)
    try:
        m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        b = O.make_bsl()
        m.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
        for k in range(1, updates + 1):
            rc = m.update(wl.H_final, 10.0 * k, b)
            if rc:
                sc = m.scalars()
                m.close()
                return rc, k, sc
        sc = m.scalars()
        m.close()
        return 0, updates, sc
    finally:
        O.set_max_rejections(0)


@pytest.mark.parametrize("precision", [0, 1])
def test_dt_min_floor_returns_fi_e_step(precision):
    """dt_min above what the tolerance needs: the first rejection that halves
    dt below it fails the update with FI_E_STEP, as in the oracle."""
    wl = _stiff(dt_min=0.3)
    rc_o, k_o, so = _oracle_until_failure(wl, 0)
    rc_g, k_g, sg = _run_until_failure(wl, 0, precision)
    assert rc_o == 3 and rc_g == _lib.FI_E_STEP
    assert k_g == k_o
    if precision == 0:
        assert sg["n_reject"] == so["n_reject"] and sg["n_accept"] == so["n_accept"]
    assert so["n_reject"] == 2   # dt 1 -> 0.5 -> 0.25 < dt_min


@pytest.mark.parametrize("precision", [0, 1])
def test_rejection_limit_returns_fi_e_step(precision):
    """More than the allowed rejections within one update: FI_E_STEP at the
    same update and after the same attempts as the oracle."""
    wl = _stiff()
    rc_o, k_o, so = _oracle_until_failure(wl, 4)
    rc_g, k_g, sg = _run_until_failure(wl, 4, precision)
    assert rc_o == 3 and rc_g == _lib.FI_E_STEP
    assert k_g == k_o
    if precision == 0:
        assert sg["n_reject"] == so["n_reject"] and sg["n_accept"] == so["n_accept"]
    assert so["n_reject"] == 5


def test_engine_barrier_wait_is_bounded(monkeypatch):
    """The step engine's grid barrier polls a bounded number of times: with
    one arrival that never comes (FI_ENGINE_BARRIER_PHANTOM, a test-only
    phantom block), every block gives up at its first barrier, the update
    fails with FI_E_TIMEOUT instead of hanging, and the device stays
    usable: a new handle then integrates normally."""
    import time
    wl = W.config2(n=128, L=3000e3 * 128 / 256, dt=1.0, stage_mode=1)

    def domain():
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
        d.set_fields(**wl.padded_fields(d.nx, d.ny))
        b = gpu_bsl()
        d.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
        return d, b

    monkeypatch.setenv("FI_ENGINE_BARRIER_PHANTOM", "1")
    d, b = domain()
    a = time.perf_counter()
    with pytest.raises(_lib.FiError) as e:
        d.update(wl.H_at(10.0), 10.0, b)
    assert e.value.code == _lib.FI_E_TIMEOUT
    assert time.perf_counter() - a < 60.0
    d.close()
    monkeypatch.delenv("FI_ENGINE_BARRIER_PHANTOM")
    d, b = domain()
    d.update(wl.H_at(10.0), 10.0, b)
    assert np.abs(d.field("w")).max() > 0
    d.close()


@pytest.mark.parametrize("dt_method", [2, 1, 0])
def test_llra_load_at_the_corners(dt_method):
    """LLRA (test1b's method) under a load covering the whole domain: the
    relaxation rate at the corners is not zero, and it must not be corrected
    by the corner mean that the LV-ELVA rate gets."""
    p = dict(P.DEFAULTS)
    p.update(method=1, dt_method=dt_method, stage_mode=0)
    n, dx = 24, 100e3
    H = 500.0 + 300.0 * np.cos(np.linspace(0, 3, n))[None, :] * np.ones((n, 1))
    wl = W.Workload(name="llra_full", params=p, nx_ice=n, ny_ice=n, dx=dx, z_bed=np.full((n, n), 1e6), H_final=H)
    dom = Domain(p, n, n, dx, precision=0)
    orc = O.Model(p, n, n, dx, dx)
    b, bo = gpu_bsl(), O.make_bsl()
    dom.init_state(wl.z_bed, np.zeros_like(H), 0.0, b)
    orc.init_state(wl.z_bed, np.zeros_like(H), 0.0, bo)
    for k in range(1, 6):
        dom.update(H, 10.0 * k, b)
        assert orc.update(H, 10.0 * k, bo) == 0
    w_g, w_o = dom.field("w"), orc.field("w")
    assert abs(w_o[0, 0]) > 0
    assert rel(w_g, w_o) <= TOL64
    dom.close()
    orc.close()


NAMELIST = """&isostasy
    method = 3
    dt_method = "tsit54"
    interactive_sealevel = .false.
    include_elastic = .true.
    heterogeneous_ssh = .true.
    lithosphere = "uniform"
    mantle = "uniform"
    zl = 88.0
    viscosities = 1e21
    E = 66.0
    nu = 0.28
    rho_uppermantle = 3400.0
    rho_litho = 3200.0
    dt_diagnostics = 10.0
    atol = 1e-2
    rtol = 1e-4
    dt_init = 1.0
    dt_max = 10.0
    pad = 0.0
/
&barysealevel
    method = "const"
    bsl_init = 0.0
    A_ocean_pd = 3.625e14
/
"""


@pytest.mark.parametrize("precision", [0, 1])
def test_reference_api_driver_loop(tmp_path, precision):
    """The reference driver's call sequence through the Python mirror of the
    Fortran API: isos_init from a namelist file, isos_init_state, then every
    dtt bsl_update and isos_update, reading isos%out; against the oracle
    driven the same way."""
    path = os.path.join(str(tmp_path), "isostasy.nml")
    with open(path, "w") as fh:
        fh.write(NAMELIST)
    n, dx = 41, 100e3
    H = W.disc(n, n, dx)
    z_bed = np.full((n, n), 1e6)
    isos, bsl = I.IsosClass(), I.BslClass()
    I.isos_init(isos, path, "isostasy", n, n, dx, dx, precision=precision)
    I.bsl_init(bsl, path, 0.0)
    I.isos_init_state(isos, z_bed, np.zeros_like(H), 0.0, bsl)
    par = P.load(path)
    orc = O.Model(par, n, n, dx, dx)
    bo = O.make_bsl()
    orc.init_state(z_bed, np.zeros_like(H), 0.0, bo)
    for k in range(1, 9):
        t = 10.0 * k
        I.bsl_update(bsl, t)
        I.isos_update(isos, H, t, bsl)
        O.lib().orc_bsl_update(bo, t)
        assert orc.update(H, t, bo) == 0
    tol = TOL64 if precision == 0 else 1e-5
    dom = isos.dom
    for f in ("z_bed", "w", "we", "dz_ss", "z_ss"):
        ref = dom.crop(orc.field(f))
        got = isos.out[f]
        assert got.shape == (n, n)
        if np.abs(ref).max() > 0:
            assert rel(got, ref) <= tol, f
    for m in MASKS:
        assert np.array_equal(isos.out[m].astype(bool), dom.crop(orc.field(m)).astype(bool)), m
    I.isos_end(isos)
    orc.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_c_driver_replays_reference_loop(tmp_path, precision):
    """The C driver (tests/driver/fi_test_isostasy.c) runs the reference's
    test loop for its disc experiment test1d through the C ABI: bsl_update
    then isos_update every dtt, isos%out read back every dt_out.  Its
    outputs against the oracle driven through the same sequence."""
    import subprocess
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "driver"))
    import build_driver
    exe = build_driver.build()
    n, dx, nt, dtt, dt_out = 41, 100e3, 31, 10.0, 100.0
    out = os.path.join(str(tmp_path), "out.bin")
    r = subprocess.run([exe, out, str(precision), str(n), repr(dx), str(nt), repr(dtt), repr(dt_out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rec = np.fromfile(out, dtype=np.float64).reshape(-1, 1 + 4 * n * n)
    assert list(rec[:, 0]) == [0.0, 100.0, 200.0, 300.0]
    p = dict(P.DEFAULTS)            # the test1d values the driver sets
    orc = O.Model(p, n, n, dx, dx)
    xc = (np.arange(n) - (n - 1) / 2.0) * dx
    H1 = np.where(xc[None, :] ** 2 + xc[:, None] ** 2 <= (1000e3) ** 2, 1000.0, 0.0)
    H0 = np.zeros_like(H1)
    z_bed = np.full((n, n), 1e6)
    bo = O.make_bsl()
    O.lib().orc_bsl_update(bo, 0.0)
    orc.init_state(z_bed, H0, 0.0, bo)
    i1, i2, j1, j2 = orc.icrop1, orc.icrop2, orc.jcrop1, orc.jcrop2
    k_out = 0
    tol = TOL64 if precision == 0 else 1e-5
    for k in range(1, nt + 1):
        t = (k - 1) * dtt
        O.lib().orc_bsl_update(bo, t)
        assert orc.update(H1 if t > 0 else H0, t, bo) == 0
        if t % dt_out == 0.0:
            got = rec[k_out, 1:].reshape(4, n, n)
            crop = lambda f: orc.field(f)[j1 - 1:j2, i1 - 1:i2]
            for i, f in enumerate(("z_bed", "w", "we")):
                ref = crop(f)
                if np.abs(ref).max() > 0 and f != "z_bed":
                    assert rel(got[i], ref) <= tol, (t, f, rel(got[i], ref))
                elif f == "z_bed":
                    assert np.abs(got[i] - ref).max() <= tol * max(np.abs(crop("w")).max(), 1.0), (t, f)
            assert np.array_equal(got[3] != 0.0, crop("maskocean") != 0), t
            k_out += 1
    assert k_out == 4
    assert np.abs(rec[-1, 1 + n * n:1 + 2 * n * n]).max() > 1.0   # the disc has depressed the bed
    orc.close()


def test_metrics_json_and_sink(tmp_path, monkeypatch):
    """fi_metrics_json reports the handle's run (updates, accepted and
    rejected steps, adaptive attempts, kernels, device status) as the
    scalars give them (attempts = accepted + rejected); with FI_METRICS_FILE set, fi_destroy appends that
    line to the file."""
    import json
    path = os.path.join(str(tmp_path), "metrics.jsonl")
    monkeypatch.setenv("FI_METRICS_FILE", path)
    wl = W.config1(48)
    wl.params["stage_mode"] = 0
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
    b = gpu_bsl()
    dom.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
    for k in range(1, 5):
        dom.update(wl.H_final, 10.0 * k, b)
    m, sc = dom.metrics(), dom.scalars()
    assert m["updates"] == 4 and m["t"] == sc["t"] == 40.0
    assert m["n_accept"] == sc["n_accept"] > 0 and m["n_reject"] == sc["n_reject"]
    assert m["n_attempt"] == m["n_accept"] + m["n_reject"]
    assert m["kernels_enqueued"] > 0 and m["status"] == 0
    assert m["precision"] == "mixed" and (m["nx"], m["ny"]) == (dom.nx, dom.ny)
    dom.close()
    with open(path) as fh:
        lines = [json.loads(v) for v in fh.read().splitlines()]
    assert lines[-1]["updates"] == 4 and lines[-1]["n_accept"] == m["n_accept"]
