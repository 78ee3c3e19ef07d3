"""GPU parity tests: libfigpu.so (through the C ABI) against the oracle.

Bars: plain FP64 form within 1e-10 of max|value| in every floating field,
masks bit-exact; mixed FP32/FP64 form within 1e-5 of max|u|.
"""
import json
import os

import numpy as np
import pytest

from fastisostasy_gb300 import _lib
from fastisostasy_gb300 import workloads as W
from fastisostasy_gb300.isostasy import Domain
from harness import Pair, gpu_bsl, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-10
TOLMIX = 1e-5


def params(name, **over):
    with open(os.path.join(GOLDEN, "params_%s.json" % name)) as fh:
        p = json.load(fh)
    p.update(over)
    return p


def random_case(nx, ny, seed, even_R):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((ny, nx)) * 100
    cf = rng.standard_normal((ny, nx)) * 1e5
    mask = (rng.random((ny, nx)) > 0.15).astype(np.uint8)
    D = 1e24 * (1 + rng.random((ny, nx)))
    eta = 1e21 * (1 + rng.random((ny, nx)))
    R = np.ones((ny, nx)) if even_R else 1 + 0.2 * rng.random((ny, nx))
    return w, cf, mask, D, eta, R


@pytest.mark.parametrize("nx,ny,even", [(16, 16, True), (32, 32, False), (64, 64, True), (128, 128, False),
                                        (122, 122, True), (48, 80, False), (256, 256, True), (192, 192, False)])
@pytest.mark.parametrize("precision", [0, 1])
def test_lvelva(nx, ny, even, precision):
    """calc_lvelva (src/lv_elva.f90:31-126) on random fields."""
    dx = 50e3
    p = params("test1d", nx_target=nx if nx != ny else 0, ny_target=ny if nx != ny else 0)
    dom = Domain(p, nx, ny, dx, precision=precision)
    assert (dom.nx, dom.ny) == (nx, ny)
    w, cf, mask, D, eta, R = random_case(nx, ny, nx * 7 + ny, even)
    dom.set_fields(D_lith=D, eta_eff=eta, R=R, maskactive=mask)
    got = dom.lvelva(w, cf)
    kap = dom.field("kappa")
    dxm = np.full((ny, nx), dx)
    ref = O.lvelva(w, cf, mask, p["g"], p["nu"], D, eta, R, kap, dxm, dxm, dom.scalars()["sec_per_year"])
    assert rel(got, ref) <= (TOL64 if precision == 0 else TOLMIX)
    dom.close()


@pytest.mark.parametrize("n", [16, 32, 64, 122, 128])
@pytest.mark.parametrize("precision", [0, 1])
def test_convolution(n, precision):
    """precomputed_fftconvolution with the elastic and geoid kernels."""
    dx = 50e3
    p = params("test2c", min_pad=0.0)
    dom = Domain(p, n, n, dx, precision=precision)
    M = 2 * n - 1
    x = np.random.default_rng(n).standard_normal((n, n)) * 1e7
    for k, G in ((0, dom.field("GE")), (1, dom.field("GN"))):
        ref = O.conv(O.kernel_spectrum(G, M), x, M)
        got = dom.convolve(k, x)
        assert rel(got, ref) <= (TOL64 if precision == 0 else TOLMIX), (k, rel(got, ref))
    # the product's Green's functions equal the oracle's restatement: GE bit
    # for bit (table interpolation, unfused products), GN to the last place
    # of the device sine
    assert np.array_equal(dom.field("GE"), O.elastic_green(n, n, dx))
    assert rel(dom.field("GN"), O.zss_green(n, n, p["m_earth"], p["r_earth"], dx)) <= 4e-16
    dom.close()


FIELDS = ["w", "we", "z_bed", "dz_ss", "dwdt", "canom_full", "z_ss", "Haf", "x"]
MASKS = ["maskocean", "maskgrounded", "maskcontinent"]


def compare(pair, tol, fields=FIELDS, masks=True):
    worst = {}
    for f in fields:
        a, b = pair.dom.field(f), pair.orc.field(f)
        worst[f] = rel(a, b) if np.abs(b).max() > 0 else float(np.abs(a).max())
        assert worst[f] <= tol, (f, worst[f])
    if masks:
        for m in MASKS:
            assert np.array_equal(pair.dom.field(m), pair.orc.field(m)), m
    return worst


def ref_disc(name, n=31, dx=200e3, **over):
    p = params(name, **over)
    H = W.disc(n, n, dx)
    return W.Workload(name=name, params=p, nx_ice=n, ny_ice=n, dx=dx, z_bed=np.full((n, n), 1e6), H_final=H)


@pytest.mark.parametrize("name,over", [("test1d", {}), ("test1e", {}), ("test2a", {}), ("test2b", {}), ("test2c", {}),
                                       ("test3a", {}), ("test3b", {}), ("test3c", {}), ("test3d", {}),
                                       ("test2c", {"lithosphere": 2})])
def test_reference_experiments_tsit54(name, over):
    """Reference experiments (par/*.nml) with the reference's own integrator
    semantics (frozen RHS, transposed Tsit5 tableau).  test2c with a
    Gaussian-thinned lithosphere makes R laterally variable (not even in the
    wavenumbers), which exercises the general Hartley-basis multiply."""
    pair = Pair(ref_disc(name, **over))
    pair.init()
    pair.step(30)
    compare(pair, TOL64)
    so, sg = pair.orc.scalars(), pair.dom.scalars()
    # identical accept/reject sequence; dt carries the error norm, whose sum
    # order differs (parallel reduction), so it agrees to rounding only
    assert so["n_accept"] == sg["n_accept"] and so["n_reject"] == sg["n_reject"]
    assert so["t"] == sg["t"] and abs(so["dt"] - sg["dt"]) <= 1e-10 * so["dt"]
    pair.close()


@pytest.mark.parametrize("name", ["test1a", "test1b", "test1c"])
@pytest.mark.parametrize("dt_method", [2, 1, 0])
@pytest.mark.parametrize("precision", [0, 1])
def test_relaxation_methods(name, dt_method, precision):
    """The reference's experiments test1a (method 0, no displacement), test1b
    (LLRA) and test1c (LV-ELRA: load convolved with the Kelvin-function
    Green's function, then relaxation over tau) with each integrator, in the
    reference's integrator semantics."""
    pair = Pair(ref_disc(name, dt_method=dt_method), precision=precision)
    pair.init()
    pair.step(12)
    if precision == 0:
        compare(pair, TOL64)
    else:
        w_o, w_g = pair.orc.field("w"), pair.dom.field("w")
        if np.abs(w_o).max() > 0:
            assert rel(w_g, w_o) <= TOLMIX
        else:
            assert np.abs(w_g).max() == 0
    pair.close()


@pytest.mark.parametrize("name,over", [("test1d", {}), ("test2c", {"lithosphere": 2}), ("test3c", {})])
@pytest.mark.parametrize("precision", [0, 1])
def test_true_stage_tsit54(name, over, precision):
    """Tsitouras 5(4) with true stages (the Dormand-Prince 5(4) pair with
    FSAL, stage states carrying the mantle term): no reference counterpart,
    GPU against the oracle's same mode."""
    pair = Pair(ref_disc(name, stage_mode=1, **over), precision=precision)
    pair.init()
    pair.step(20)
    if precision == 0:
        compare(pair, TOL64)
        so, sg = pair.orc.scalars(), pair.dom.scalars()
        assert so["n_accept"] == sg["n_accept"] and so["n_reject"] == sg["n_reject"]
        assert so["t"] == sg["t"] and abs(so["dt"] - sg["dt"]) <= 1e-10 * so["dt"]
    else:
        w_o, w_g = pair.orc.field("w"), pair.dom.field("w")
        assert rel(w_g, w_o) <= TOLMIX
    pair.close()


@pytest.mark.parametrize("dt_method,stage_mode", [(1, 0), (1, 1), (0, 0), (0, 1)])
def test_config2_rk4_euler(dt_method, stage_mode):
    wl = W.config2(n=64, L=3000e3 * 64 / 256, dt=1.0, stage_mode=stage_mode)
    wl.params["dt_method"] = dt_method
    pair = Pair(wl)
    pair.init()
    pair.step(6)
    compare(pair, TOL64)
    pair.close()


def test_config3_interactive_sealevel_rectangular():
    """Interactive sea level, masks, elastic + geoid, two-layer freqdomain
    lumping (non-even R -> general Hartley path), rectangular padding."""
    wl = W.config3(nx_ice=40, ny_ice=72, dx=20e3, nx_pad=64, ny_pad=96)
    pair = Pair(wl)
    pair.init()
    pair.step(8)
    compare(pair, TOL64)
    assert pair.dom.field("R").std() > 0
    pair.close()


def test_mixed_precision_error_bound():
    wl = W.config2(n=64, L=3000e3 * 64 / 256, dt=1.0, stage_mode=1)
    a = Pair(wl, precision=0)
    b = Pair(wl, precision=1, gpu=True)
    a.init(); b.init()
    a.step(20); b.step(20)
    w64, w32 = a.dom.field("w"), b.dom.field("w")
    assert rel(w32, w64) <= TOLMIX
    a.close(); b.close()


@pytest.mark.parametrize("precision,n", [(0, 32), (1, 64)])
def test_outputs_and_restart_roundtrip(precision, n):
    """isos%out of fi_update equals the fields; a restart (state export,
    further updates, import) repeats an update bit for bit — in the mixed
    form through the step engine, whose row flags restart with the state."""
    wl = W.config2(n=n, L=3000e3 * n / 256, dt=1.0, stage_mode=1)
    pair = Pair(wl, precision=precision)
    pair.init()
    pair.step(3)
    dom = pair.dom
    buf = dom.state_export()
    ni = (wl.ny_ice, wl.nx_ice)
    out = {k: np.zeros(ni) for k in ("z_bed", "w", "we", "dz_ss")}
    out["maskocean"] = np.zeros(ni, dtype=np.uint8)
    t = pair.t + wl.dtt
    dom.update(wl.H_at(t), t, pair.bg, out=out)
    assert np.array_equal(out["w"], dom.crop(dom.field("w")))
    assert np.array_equal(out["z_bed"], dom.crop(dom.field("z_bed")))
    w1 = dom.field("w")
    dom.update(wl.H_at(t + wl.dtt), t + wl.dtt, pair.bg)   # advance further before the restart
    dom.state_import(buf)
    dom.update(wl.H_at(t), t, pair.bg)
    assert np.array_equal(dom.field("w"), w1)
    pair.close()


def test_page_locked_and_pageable_host_arrays_agree():
    """fi_update on a grid above 65536 ice cells (one copy per field):
    outputs into page-locked arrays go straight from the device, pageable
    ones through the staging buffer, absent ones are skipped; a page-locked
    ice load is uploaded directly.  Every output equals the field, and the
    two input forms give the same state bit for bit."""
    import torch
    wl = W.config2(n=512, L=512 * 11.71875e3, dt=1.0, stage_mode=1)
    ni = (wl.ny_ice, wl.nx_ice)
    res = []
    for pin in (False, True):
        dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
        dom.set_fields(**wl.padded_fields(dom.nx, dom.ny))
        bg = gpu_bsl()
        dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)

        def arr(dtype, locked):
            if locked:
                return torch.zeros(ni, dtype=dtype, pin_memory=True).numpy()
            return np.zeros(ni, dtype=np.float64 if dtype == torch.float64 else np.uint8)

        # page-locked and pageable outputs side by side; dwdt and Hice absent
        out = {"w": arr(torch.float64, pin), "we": arr(torch.float64, not pin),
               "z_bed": arr(torch.float64, pin), "z_ss": arr(torch.float64, True),
               "dz_ss": arr(torch.float64, False), "canom_full": arr(torch.float64, pin),
               "maskocean": arr(torch.uint8, pin), "maskgrounded": arr(torch.uint8, not pin),
               "maskcontinent": arr(torch.uint8, True)}
        H = arr(torch.float64, pin)
        for t in (10.0, 20.0):
            H[...] = wl.H_at(t)
            dom.update(H, t, bg, out=out)
        for k in ("w", "we", "z_bed", "z_ss", "dz_ss", "canom_full"):
            assert np.array_equal(out[k], dom.crop(dom.field(k))), k
        for k in ("maskocean", "maskgrounded", "maskcontinent"):
            assert np.array_equal(out[k], dom.crop(dom.field(k)).astype(np.uint8)), k
        res.append(dom.field("w"))
        dom.close()
    assert np.abs(res[0]).max() > 0
    assert np.array_equal(res[0], res[1])


def test_error_status_codes():
    wl = W.config2(n=32, L=3000e3 * 32 / 256, dt=1.0, stage_mode=1)
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx)
    bg = gpu_bsl()
    with pytest.raises(_lib.FiError) as e:
        dom.update(wl.H_at(10.0), 10.0, bg)
    assert e.value.code == _lib.FI_E_STATE
    dom.set_fields(**wl.padded_fields(dom.nx, dom.ny))
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)
    H = wl.H_at(10.0).copy()
    H[3, 3] = np.nan
    with pytest.raises(_lib.FiError) as e:
        dom.update(H, 10.0, bg)
    assert e.value.code == _lib.FI_E_NAN
    dom.close()
    # dt = 10 yr on an 11.7 km grid with D ~ 2e25 diverges (lambda*dt ~ -18);
    # the domain must be wider than the disc so that its edge seeds short waves
    wl = W.config2(n=128, L=3000e3 * 128 / 256, dt=10.0, stage_mode=1)
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx)
    dom.set_fields(**wl.padded_fields(dom.nx, dom.ny))
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)
    with pytest.raises(_lib.FiError) as e:
        for k in range(1, 10):
            dom.update(wl.H_at(10.0 * k), 10.0 * k, bg)
    assert e.value.code == _lib.FI_E_LARGE
    dom.close()


@pytest.mark.parametrize("precision,integrator", [(0, "rk4"), (1, "rk4"), (0, "tsit54"), (1, "tsit54"),
                                                 (0, "tsit54-true"), (1, "tsit54-true")])
def test_graph_replay_matches_eager(precision, integrator, monkeypatch):
    """Updates replayed from a captured CUDA graph give bit-identical state to
    the same updates launched one kernel at a time.  For Tsit5 the captured
    graph decides accept/reject on the device (WHILE node) where the eager
    path decides on the host: same attempts, same bits."""
    if integrator == "rk4":
        wl = W.config2(n=64, L=3000e3 * 64 / 256, dt=1.0, stage_mode=1)
    elif integrator == "tsit54":
        wl = ref_disc("test1d")
    else:
        wl = ref_disc("test1d", stage_mode=1)
    out = []
    for no_graph in ("1", "0"):
        monkeypatch.setenv("FI_NO_GRAPHS", no_graph)
        p = Pair(wl, precision=precision)
        p.init()
        p.step(8)
        sc = p.dom.scalars()
        out.append((p.dom.field("w"), p.dom.field("z_bed"), p.dom.field("we"), p.dom.field("dwdt"),
                    np.array([sc["t"], sc["dt"], sc["n_accept"], sc["n_reject"], sc["n_rhs"]])))
        p.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision,n", [(0, 128), (0, 256), (1, 128), (1, 256)])
def test_step_engine_matches_kernel_sequence(precision, n, monkeypatch):
    """The cooperative RK4 step engine against the one-kernel-per-pass path:
    FP64 to rounding, mixed within the mixed-form bound."""
    wl = W.config2(n=n, L=3000e3 * n / 256, dt=1.0, stage_mode=1)
    res = []
    for no_engine in ("1", "0"):
        monkeypatch.setenv("FI_NO_ENGINE", no_engine)
        p = Pair(wl, precision=precision)
        p.init()
        p.step(5)
        res.append(p.dom.field("w"))
        if no_engine == "0" and precision == 0:
            compare(p, TOL64)
        p.close()
    assert rel(res[1], res[0]) <= (1e-12 if precision == 0 else 1e-6)


def test_step_engine_shapes_agree_bit_for_bit(monkeypatch):
    """512^2 mixed: the four-row engine shape (one 1024-thread block per SM,
    power-of-two transforms) and the two-row shape run the same arithmetic
    per cell, so they agree bit for bit; both match the kernel sequence
    within the mixed-form bound."""
    wl = W.config2(n=512, L=3000e3 * 2, dt=1.0, stage_mode=1)
    res = {}
    for key, env in (("ra4", {}), ("ra2", {"FI_ENGINE_RA": "2"}), ("seq", {"FI_NO_ENGINE": "1"})):
        monkeypatch.delenv("FI_ENGINE_RA", raising=False)
        monkeypatch.delenv("FI_NO_ENGINE", raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
        assert dom.ny <= 600, "the step engine runs only where its stencil phase fits one wave"
        f = wl.padded_fields(dom.nx, dom.ny)
        if f:
            dom.set_fields(**f)
        m = wl.bsl.get("method", 0)
        bg = gpu_bsl(m, wl.bsl.get("bsl_init", 0.0), wl.bsl.get("A_ocean_pd", 3.625e14))
        dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)
        t = 0.0
        for _ in range(3):
            t += wl.dtt
            _lib.load().fi_bsl_update(bg, t)
            dom.update(wl.H_at(t), t, bg)
        res[key] = dom.field("w")
        dom.close()
    assert np.abs(res["ra4"]).max() > 0
    assert np.array_equal(res["ra4"], res["ra2"])
    assert rel(res["ra4"], res["seq"]) <= 1e-6


def test_device_analytical_disk():
    """fi_elva_disk (the analytical ELVA disc evaluated on the device) against
    the oracle's evaluation of the same integral, then used as the validator
    of a GPU run of the reference's disc experiment test1d."""
    from oracle import analytical as A
    import ctypes as C
    L = _lib.load()
    n, dx, T = 61, 100e3, 3000.0
    p = params("test1d")
    D = p["E"] * 1e9 * p["zl"][0] ** 3 / (12.0 * (1.0 - p["nu"] ** 2))
    got = np.zeros((n, n))
    rc = L.fi_elva_disk(n, n, dx, 1000e3, 1000.0, 1e21, D, 910.0, 3400.0, 9.81, T,
                        got.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    ana = A.elva_disk(n, n, dx, 1000e3, 1000.0, 1e21, D, 910.0, 3400.0, 9.81, T)
    assert rel(got, ana) <= 1e-9
    # the GPU solution of test1d against it (the oracle's own physics check)
    xc = -3000e3 + dx * np.arange(n)
    H = np.where(xc[None, :] ** 2 + xc[:, None] ** 2 <= 1000e3 ** 2, 1000.0, 0.0)
    dom = Domain(p, n, n, dx)
    b = gpu_bsl()
    dom.init_state(np.full((n, n), 1e6), np.zeros_like(H), 0.0, b)
    out = {"z_bed": np.zeros((n, n))}
    for k in range(1, int(T / 10) + 2):
        t = (k - 1) * 10.0
        dom.update(H if t > 0 else np.zeros_like(H), t, b, out=out)
    dom.close()
    zb = out["z_bed"] - 1e6
    assert abs(zb.min() - got.min()) <= 0.03 * abs(got.min())


def _tsit_run(wl, precision, eta_scale=1.0, times=(10.0, 20.0, 30.0, 40.0)):
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
    f = wl.padded_fields(dom.nx, dom.ny)
    if "eta_eff" in f:
        f["eta_eff"] = f["eta_eff"] * eta_scale
    if f:
        dom.set_fields(**f)
    b = gpu_bsl()
    dom.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
    for t in times:
        dom.update(wl.H_final, t, b)
    w = dom.field("w")
    dom.close()
    return w


@pytest.mark.parametrize("member", [None, 7, 3])
def test_mixed_reference_tsit54_against_fp64(member):
    """Reference-compatible Tsit5 in the mixed form (now%w as a float pair,
    column-strip stencil, one-pass error norm) against the FP64 form over a
    few coupling steps: within the mixed-form bound."""
    if member is None:
        wl = W.config1(56)
        wl.params["stage_mode"] = 0
    else:
        wl = W.ensemble_member(member, stage_mode=0)
    assert rel(_tsit_run(wl, 1), _tsit_run(wl, 0)) <= TOLMIX


def test_reference_tsit54_stability_edge_sensitivity():
    """The reference's Tsit5 evaluates one RHS per attempt (every stage
    takes k(x)), so x2 is a forward-Euler step and the error estimate
    0.2 dt |k| bounds the increment, not the stability of the stiff modes.
    On a stiff member (384^2, eta down to ~1e20) the accepted steps ride the
    stability edge and the FP64 form itself moves by far more than 1e-5 of
    max|w| when eta changes by 1e-12: no precision can be held to the mixed
    bound there, which is why the bound above is checked on members off
    that edge."""
    wl = W.ensemble_member(2, stage_mode=0)
    assert rel(_tsit_run(wl, 0, eta_scale=1.0 + 1e-12), _tsit_run(wl, 0)) > 1e-3


def _rheo_file(nx_dom, dx, seed, nz=5):
    """A synthetic rheology file: a coarser grid than the domain (its edges
    inside the domain, so the flat extension is exercised), thickness in km,
    log10 eta with values beyond the [16, 23] clamp, a stddev field."""
    rng = np.random.default_rng(seed)
    L = nx_dom * dx / 2
    xr = np.linspace(-0.9 * L, 0.9 * L, 23)
    yr = np.linspace(-0.85 * L, 0.95 * L, 19)
    X, Y = np.meshgrid(xr, yr)
    thick = 90.0 + 30.0 * np.sin(X / 4e5) * np.cos(Y / 5e5) + rng.random(X.shape)
    zr = np.array([-660e3, -410e3, -250e3, -120e3, 0.0])
    lg = np.stack([20.5 + 0.3 * k + 0.8 * np.sin((X + k * 1e5) / 3e5) * np.cos(Y / 4e5) for k in range(nz)])
    lg[0, :3, :3] = 24.0
    lg[-1, -2:, -2:] = 15.0
    sd = 0.1 + 0.05 * rng.random(lg.shape)
    return xr, yr, zr, thick, lg, sd


@pytest.mark.parametrize("radius,stddev,lumping,layering", [(0.0, False, 5, 1), (120e3, True, 5, 0),
                                                             (120e3, False, 4, 1), (0.0, True, 0, 1)])
def test_rheology_file(radius, stddev, lumping, layering):
    """The rheology_file branches of isos_init on the device (fi_set_rheology:
    bilinear onto the grid, smooth_gauss_2D, clamp, depth interpolation,
    lumping, scaling) against the oracle's step-by-step restatement, then a
    few updates with those fields against the oracle."""
    wl = W.config1(48)
    wl.t_end = 30.0
    wl.params.update(nl=3, zl=[100e3, 250e3, 500e3], viscosities=[1e21, 1e21, 1e21], lumping=lumping,
                     layering=layering, dl=120e3, mantle=3, lithosphere=3, correct_compression=1,
                     visc_scaling_method=0 if stddev else 1, viscosity_scaling=1.5)
    pair = Pair(wl)
    dom, orc = pair.dom, pair.orc
    nx, ny, dx = dom.nx, dom.ny, wl.dx
    xc = (np.arange(1, nx + 1) - nx // 2 - 1) * dx
    yc = (np.arange(1, ny + 1) - ny // 2 - 1) * dx
    xr, yr, zr, thick, lg, sd = _rheo_file(nx, dx, 5)
    dom.set_rheology(xr, yr, zr, litho_thickness=thick, litho_thickness_scaling=1e3, log10_viscosity=lg,
                     stddev_log10_viscosity=sd, stddev_scaling=stddev, rheo_smoothing_radius=radius)
    cc = 1.5 / (1 + wl.params["nu"])
    He, D, eta, R = O.rheology_file(wl.params, xc, yc, dx, dom.field("kappa"), np.full((ny, nx), 100e3), xr, yr,
                                    zr, thick, 1e3, lg, sd, stddev, radius, cc)
    assert rel(dom.field("D_lith"), D) <= 1e-12
    assert rel(dom.field("eta_eff"), eta) <= 1e-12
    assert rel(dom.field("R"), R) <= 1e-12
    if lumping == 5:
        assert R.std() > 0
    orc.set_fields(D_lith=D, eta_eff=eta, R=R)
    pair.init()
    pair.step(3)
    compare(pair, TOL64)
    pair.close()


def test_rheology_file_rejects_a_window_wider_than_the_grid():
    wl = W.config1(32)
    wl.params.update(mantle=3, lithosphere=3)
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=0)
    xr, yr, zr, thick, lg, sd = _rheo_file(dom.nx, wl.dx, 1)
    with pytest.raises(Exception):
        dom.set_rheology(xr, yr, zr, litho_thickness=thick, litho_thickness_scaling=1e3,
                         rheo_smoothing_radius=40 * wl.dx)
    dom.close()


def test_async_output_snapshots_match_synchronous_outputs():
    """fi_output_async snapshots taken between asynchronous updates (copied
    on a side stream while the next updates run) equal the isos%out fields
    that synchronous fi_update calls return at the same times."""
    import torch
    from fastisostasy_gb300.isostasy import OUT_FIELDS, OUT_MASKS
    wl = W.config2(n=64, L=3000e3 * 64 / 256, dt=1.0, stage_mode=1)
    times = [wl.dtt * (k + 1) for k in range(6)]
    # synchronous: outputs of fi_update every second update
    a = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
    ba = gpu_bsl()
    a.init_state(wl.z_bed, wl.H_at(0.0), 0.0, ba)
    want = []
    for k, t in enumerate(times):
        out = None
        if k % 2 == 1:
            out = {f: np.zeros((wl.ny_ice, wl.nx_ice)) for f in OUT_FIELDS}
            out.update({m: np.zeros((wl.ny_ice, wl.nx_ice), dtype=np.uint8) for m in OUT_MASKS})
        a.update(wl.H_final, t, ba, out)
        if out is not None:
            want.append(out)
    a.close()
    # asynchronous: device-resident updates, a snapshot after every second one
    b = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
    bb = gpu_bsl()
    b.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bb)
    H = torch.from_numpy(np.ascontiguousarray(wl.H_final)).to("cuda")
    nb = b.output_bytes() // 8
    bufs = [torch.empty(nb, dtype=torch.float64).pin_memory() for _ in range(len(want))]
    j = 0
    for k, t in enumerate(times):
        b.update_async(H.data_ptr(), t, bb)
        if k % 2 == 1:
            b.output_async(bufs[j].data_ptr())
            j += 1
    b.output_wait()
    b.synchronize()
    for w_out, buf in zip(want, bufs):
        got = b.unpack_output(buf.numpy())
        for f in OUT_FIELDS:
            assert np.array_equal(got[f], w_out[f]), f
        for m in OUT_MASKS:
            assert np.array_equal(got[m], w_out[m].astype(bool)), m
    b.close()


def test_caller_stream():
    """fi_set_stream: the same updates on a stream the caller owns give the
    same bits as on the handle's own stream."""
    import torch
    wl = W.config2(n=48, L=3000e3 * 48 / 256, dt=1.0, stage_mode=1)
    res = []
    for use_caller in (False, True):
        dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
        dom.set_fields(**wl.padded_fields(dom.nx, dom.ny))
        b = gpu_bsl()
        dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
        st = torch.cuda.Stream() if use_caller else None
        if st is not None:
            assert dom.L.fi_set_stream(dom.h, st.cuda_stream) == 0
            assert dom.L.fi_stream(dom.h) == st.cuda_stream
        for t in (10.0, 20.0, 30.0):
            dom.update(wl.H_at(t), t, b)
        res.append(dom.field("w"))
        if st is not None:
            assert dom.L.fi_set_stream(dom.h, None) == 0
        dom.close()
    assert np.array_equal(res[0], res[1])
