"""CPU tests: the oracle against transform definitions, an independent numpy
restatement, the analytical ELVA disk and the committed golden vectors."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import np_restatement as R
from oracle import analytical as A
from fastisostasy_gb300 import workloads as W
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 12, 61, 64, 73, 122, 243, 256, 511, 1023, 1024])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert np.abs(O.cfft(x, -1) - np.fft.fft(x)).max() <= 2e-15 * np.abs(np.fft.fft(x)).max() * max(1, np.log2(n))
    assert np.abs(O.cfft(x, +1) - n * np.fft.ifft(x)).max() <= 2e-15 * n * np.abs(np.fft.ifft(x)).max() * max(1, np.log2(n))


@pytest.mark.parametrize("shape", [(8, 8), (16, 16), (12, 20), (30, 30)])
def test_dht_matches_cas_definition(shape):
    a = np.random.default_rng(1).standard_normal(shape)
    h = O.dht2d(a)
    ref = R.dht2d(a)
    assert np.abs(h - ref).max() <= 1e-13 * np.abs(ref).max()
    # DHT is its own inverse up to N
    assert np.abs(O.dht2d(h) / a.size - a).max() <= 1e-13


@pytest.mark.parametrize("kind", ["x", "y", "xx", "yy"])
def test_derivatives_bit_exact(kind):
    rng = np.random.default_rng(2)
    u = rng.standard_normal((10, 14))
    d = 1 + rng.random((10, 14))
    f = {"x": R.d_x, "y": R.d_y, "xx": R.d_xx, "yy": R.d_yy}[kind]
    assert np.array_equal(O.derivative(kind, u, d), f(u, d))


def test_kappa_within_one_ulp():
    # the reference takes (p*p + q*q)**0.5 (pow); numpy's sqrt may differ in the last bit
    for nx, ny in [(20, 12), (64, 64), (122, 122)]:
        a, b = O.kappa(nx, ny, 1e4, 1e4), R.kappa(nx, ny, 1e4, 1e4)
        assert np.all(np.abs(a - b) <= 2.3e-16 * np.abs(b))


@pytest.mark.parametrize("n", [8, 16, 32])
def test_convolution_is_linear_convolution(n):
    rng = np.random.default_rng(n)
    ker, inp = rng.standard_normal((n, n)), rng.standard_normal((n, n))
    M = 2 * n - 1
    out = O.conv(O.kernel_spectrum(ker, M), inp, M)
    ref = R.linear_conv_crop(ker, inp)
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("n,even", [(16, True), (32, False), (24, False)])
def test_lvelva_matches_numpy_restatement(n, even):
    rng = np.random.default_rng(n)
    dx = 5e4
    w = rng.standard_normal((n, n)) * 100
    cf = rng.standard_normal((n, n)) * 1e5
    mask = rng.random((n, n)) > 0.2
    D = 1e24 * (1 + rng.random((n, n)))
    eta = 1e21 * (1 + rng.random((n, n)))
    Rr = np.ones((n, n)) if even else 1 + 0.1 * rng.random((n, n))
    kap = O.kappa(n, n, dx, dx)
    dxm = np.full((n, n), dx) * (1 + 0.01 * rng.random((n, n)))
    a = O.lvelva(w, cf, mask, 9.81, 0.28, D, eta, Rr, kap, dxm, dxm.copy(), 31557600.0)
    b = R.lvelva(w, cf, mask, 9.81, 0.28, D, eta, Rr, kap, dxm, dxm.copy(), 31557600.0)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_analytical_disk_pins_oracle():
    """Reference experiment test1d (par/test_isostasy_test1d.nml) on a 100 km
    grid against the Bueler et al. (2007) solution the reference itself
    writes as err_z_bed (src/isostasy_io.f90:382-390)."""
    with open(os.path.join(GOLDEN, "params_test1d.json")) as fh:
        p = json.load(fh)
    dx, n = 100e3, 61
    xc = -3000e3 + dx * np.arange(n)
    H = np.where(xc[None, :] ** 2 + xc[:, None] ** 2 <= 1000e3 ** 2, 1000.0, 0.0)
    m = O.Model(p, n, n, dx, dx)
    b = O.make_bsl()
    m.init_state(np.full((n, n), 1e6), np.zeros_like(H), 0.0, b)
    T = 3000.0
    for k in range(1, int(T / 10) + 2):
        t = (k - 1) * 10.0
        assert m.update(H if t > 0 else np.zeros_like(H), t, b) == 0
    zb = m.crop(m.field("z_bed")) - 1e6
    ana = A.elva_disk(n, n, dx, 1000e3, 1000.0, 1e21, m.field("D_lith")[0, 0], 910.0, 3400.0, 9.81, T)
    centre_err = abs(zb.min() - ana.min()) / abs(ana.min())
    rms_err = np.sqrt(np.mean((zb - ana) ** 2)) / abs(ana.min())
    assert centre_err < 0.03, centre_err
    assert rms_err < 0.05, rms_err


def test_golden_vectors():
    """Regression pin: oracle outputs committed by tests/golden/make_golden.py."""
    path = os.path.join(GOLDEN, "oracle_golden.npz")
    g = np.load(path)
    import make_golden_cases as MG
    for name, fn in MG.CASES.items():
        out = fn()
        for k, v in out.items():
            key = name + "__" + k
            assert key in g.files, key
            ref = g[key]
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(v - ref).max() <= 1e-12 * scale, key


def test_kei_table_matches_reference_table():
    """The Kelvin-function table of LV-ELRA, rebuilt from kei itself, equals
    the reference's tabulated values (src/kelvin_function.f90, read into
    tests/golden/kei_reference.npz by tests/golden/make_golden.py) bit for
    bit after the same rounding."""
    ref = np.load(os.path.join(GOLDEN, "kei_reference.npz"))
    rn, kv = np.zeros(1001), np.zeros(1001)
    dp = C.POINTER(C.c_double)
    O.lib().orc_kei_table(rn.ctypes.data_as(dp), kv.ctypes.data_as(dp))
    assert np.array_equal(rn, ref["rn"]) and np.array_equal(kv, ref["kei"])


def _relax_run(name, T, dt_save=None, n=41, dx=100e3):
    with open(os.path.join(GOLDEN, "params_%s.json" % name)) as fh:
        p = json.load(fh)
    xc = -(n // 2) * dx + dx * np.arange(n)
    H = np.where(xc[None, :] ** 2 + xc[:, None] ** 2 <= 1000e3 ** 2, 1000.0, 0.0)
    m = O.Model(p, n, n, dx, dx)
    b = O.make_bsl()
    m.init_state(np.full((n, n), 1e6), np.zeros_like(H), 0.0, b)
    for k in range(1, int(T / 10) + 1):
        assert m.update(H, k * 10.0, b) == 0
    w = m.crop(m.field("w"))
    load = m.crop(m.field("canom_load"))
    m.close()
    return p, w, load


def test_llra_relaxes_exponentially():
    """LLRA (test1b): w = w_eq (1 - exp(-t / tau)) with w_eq = -canom_load / rho_m
    under a load switched on at t = 0 (the corner BC subtracts the corner
    mean, which is zero far from the disc)."""
    p, w, load = _relax_run("test1b", 3000.0)
    weq = -load / p["rho_uppermantle"]
    ana = weq * (1.0 - np.exp(-3000.0 / p["tau"]))
    assert np.abs(w - ana).max() <= 5e-3 * np.abs(weq).max()


def test_elra_equilibrium_matches_local_under_a_broad_load():
    """LV-ELRA (test1c): under a disc much wider than the flexural length the
    relaxed deflection at the disc centre approaches the local (LLRA)
    equilibrium -rho_i H / rho_m."""
    p, w, load = _relax_run("test1c", 30000.0)
    weq_local = -load / p["rho_uppermantle"]
    c = w.shape[0] // 2
    assert abs(w[c, c] - weq_local[c, c]) <= 0.05 * abs(weq_local[c, c])


def test_smooth_gauss_2d_keeps_constants_and_rejects_wide_windows():
    """smooth_gauss_2D's normalised window leaves a constant field unchanged
    (mirror extension included) and the reference stops when the window
    reaches past the mirrored band."""
    v = np.full((20, 24), 3.25)
    s = O.smooth_gauss_2d(v, 10e3, 35e3)
    assert np.allclose(s, 3.25, rtol=0, atol=1e-14)
    assert O.smooth_gauss_2d(v, 10e3, 120e3) is None


def test_bilinear_array_nodes_and_flat_extension():
    """bilinear_interpolation reproduces the grid values at interior nodes
    (to single precision) and holds the edge values beyond the grid."""
    xr = np.linspace(-1e6, 1e6, 21)
    yr = np.linspace(-8e5, 8e5, 17)
    z = np.random.default_rng(3).random((17, 21))
    got = O.bilinear_array(xr, yr, z, xr[3:-3], yr[3:-3])
    assert np.allclose(got, z[3:-3, 3:-3].astype(np.float32), rtol=0, atol=2e-6)
    far = O.bilinear_array(xr, yr, z, np.array([-2e6, 2e6]), np.array([-2e6, 2e6]))
    assert far[0, 0] == np.float32(z[0, 0]) and far[1, 1] == np.float32(z[-1, -1])


def test_elastic_green_uses_the_reference_table():
    """The oracle's elastic Green's function equals calc_elastic_green
    evaluated from the reference's own Farrell table (rn_vals, ge_vals of
    src/green_functions.f90, extracted into ge_reference.npz), bit for bit."""
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "ge_reference.npz"))
    rn, ge = ref["rn"], ref["ge"]
    n, dx = 24, 75e3
    got = O.elastic_green(n, n, dx)
    mx = n // 2
    f12, f981 = float(np.float32(1.e-12)), float(np.float32(9.81))
    want = np.zeros((n, n))
    for j in range(n):
        for i in range(n):
            x, y = (i - mx) * dx, (j - mx) * dx
            r = np.sqrt(x * x + y * y)
            if r > rn[41]:
                g = 0.0
            else:
                k = 0
                while k < 41 and not (rn[k] <= r < rn[k + 1]):
                    k += 1
                k = min(k, 40)
                g = ge[k] + (r - rn[k]) / (rn[k + 1] - rn[k]) * (ge[k + 1] - ge[k])
            want[j, i] = g * f12 * (dx * dx) / (f981 * max(r, dx))
    assert np.array_equal(got, want)


def test_config3_reference_tsit54_is_ill_conditioned():
    """Configuration 3 (512 x 1024, a 1e20 Pa s layer at 5 km spacing) under
    the reference's Tsit5 (frozen RHS: every attempt is a forward-Euler step,
    src/integrators.f90:131-203, src/fastisostasy.f90:677-729): a 1e-13
    relative change of the upper-mantle viscosity, far below any FP64
    implementation difference, moves w by more than 1e-3 of max|w| within
    five model years (the accept/reject counts may still coincide).  No build of
    the reference (another compiler, another CPU, FFTW) can reproduce its
    step sequence over a 10-yr coupling step; GPU parity at this size is
    therefore checked over the first two years (test_gpu_full_size.py)."""
    O.set_threads(os.cpu_count() or 1)
    O.set_reuse_frozen(True)
    try:
        out = []
        for pert in (0.0, 1e-13):
            wl = W.config3()
            wl.params["viscosities"] = [1e20 * (1 + pert), 1e21]
            m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
            b = O.make_bsl()
            m.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
            for t in (1.0, 2.0, 3.0, 4.0, 5.0):
                assert m.update(wl.H_at(t), t, b) == 0
            s = m.scalars()
            out.append((s["n_accept"], s["n_reject"], m.field("w")))
            m.close()
    finally:
        O.set_reuse_frozen(False)
    (a0, r0, w0), (a1, r1, w1) = out
    assert a0 + r0 > 100
    assert np.abs(w1 - w0).max() > 1e-3 * np.abs(w0).max()
