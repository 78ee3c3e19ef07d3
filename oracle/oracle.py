"""ctypes wrapper around the CPU FP64 oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  Fields are numpy arrays of shape
``(ny, nx)`` in C order, which is the reference's Fortran ``(nx, ny)``
column-major layout (x fastest).
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None

FIELDS = {
    "z_bed": 0, "dwdt": 1, "w": 2, "we": 3, "Haf": 4, "Hice": 5, "z_ss": 6, "dz_ss": 7,
    "canom_load": 8, "canom_full": 9, "mass_anom": 10, "maskocean": 11, "maskgrounded": 12,
    "maskcontinent": 13, "canom_mantle": 14, "canom_litho": 15, "canom_seawater": 16,
    "canom_ice": 17, "x": 18, "kappa": 19, "D_lith": 20, "eta_eff": 21, "R": 22,
    "maskactive": 23, "GE": 24, "GN": 25, "w_ref": 26, "z_bed_ref": 27, "Haf_ref": 28,
    "z_ss_ref": 29, "He_lith": 30,
}


class OrcParams(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("interactive_sealevel", C.c_int32), ("include_elastic", C.c_int32),
        ("heterogeneous_ssh", C.c_int32), ("correct_compression", C.c_int32),
        ("lithosphere", C.c_int32), ("mantle", C.c_int32), ("layering", C.c_int32),
        ("lumping", C.c_int32), ("visc_scaling_method", C.c_int32), ("nl", C.c_int32),
        ("dt_method", C.c_int32), ("stage_mode", C.c_int32), ("nx_target", C.c_int32),
        ("ny_target", C.c_int32), ("pad_", C.c_int32),
        ("dt_diagnostics", C.c_double), ("min_pad", C.c_double), ("viscosity_scaling", C.c_double),
        ("zl", C.c_double * 8), ("viscosities", C.c_double * 8), ("dl", C.c_double),
        ("eta_ref", C.c_double), ("E", C.c_double), ("nu", C.c_double), ("rho_water", C.c_double),
        ("rho_ice", C.c_double), ("rho_seawater", C.c_double), ("rho_uppermantle", C.c_double),
        ("rho_litho", C.c_double), ("g", C.c_double), ("r_earth", C.c_double),
        ("m_earth", C.c_double), ("atol", C.c_double), ("rtol", C.c_double),
        ("dt_min", C.c_double), ("dt_max", C.c_double), ("dt_init", C.c_double), ("q", C.c_double), ("tau", C.c_double),
    ]


class OrcBsl(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("constant_ocean_surface", C.c_int32), ("n_series", C.c_int32),
        ("n_aocean", C.c_int32), ("bsl_init", C.c_double), ("bsl_now", C.c_double),
        ("A_ocean_now", C.c_double), ("A_ocean_pd", C.c_double), ("time", C.c_double),
        ("series_t", C.POINTER(C.c_double)), ("series_v", C.POINTER(C.c_double)),
        ("bsl_vec", C.POINTER(C.c_double)), ("aocean_vec", C.POINTER(C.c_double)),
    ]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        u8 = C.POINTER(C.c_uint8)
        L.orc_cfft.argtypes = [C.c_int, dp, dp, C.c_int]
        L.orc_dht2d.argtypes = [C.c_int, C.c_int, dp, dp]
        L.orc_kappa.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_lvelva.argtypes = [dp, dp, dp, u8, C.c_double, C.c_double, dp, dp, dp, dp,
                                 C.c_int, C.c_int, dp, dp, C.c_double]
        L.orc_kernel_spectrum.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp]
        L.orc_conv.argtypes = [dp, C.c_int, C.c_int, C.c_int, dp, dp, dp]
        L.orc_elastic_green.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_zss_green.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double]
        for nm in ("orc_derivative_x", "orc_derivative_y", "orc_derivative_xx", "orc_derivative_yy"):
            getattr(L, nm).argtypes = [dp, dp, dp, C.c_int, C.c_int]
        L.orc_create.argtypes = [C.POINTER(OrcParams), C.c_int, C.c_int, C.c_double, C.c_double, dp]
        L.orc_create.restype = C.c_void_p
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.orc_set_fields.argtypes = [C.c_void_p, dp, dp, dp, u8]
        L.orc_init_ref.argtypes = [C.c_void_p, dp, dp, C.c_double, dp]
        L.orc_init_state.argtypes = [C.c_void_p, dp, dp, C.c_double, C.POINTER(OrcBsl)]
        L.orc_update.argtypes = [C.c_void_p, dp, C.c_double, C.POINTER(OrcBsl)]
        L.orc_bsl_update.argtypes = [C.POINTER(OrcBsl), C.c_double]
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, dp]
        L.orc_get_scalars.argtypes = [C.c_void_p, dp]
        L.orc_rhs_now.argtypes = [C.c_void_p, dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_reuse_frozen.argtypes = [C.c_int]
        L.orc_set_max_rejections.argtypes = [C.c_long]
        L.orc_set_smooth_convolution.argtypes = [C.c_int]
        L.orc_set_rhs_noise.argtypes = [C.c_double, C.c_ulonglong]
        L.orc_bilinear_array.argtypes = [dp, C.c_int, dp, C.c_int, dp, dp, C.c_int, dp, C.c_int, dp]
        L.orc_interp_0d.argtypes = [dp, dp, C.c_int, C.c_double]
        L.orc_interp_0d.restype = C.c_double
        L.orc_smooth_gauss_2d.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_smooth_gauss_2d.restype = C.c_int
        L.orc_lump3.argtypes = [dp, dp, dp, C.c_int, C.c_int, C.c_int, dp, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def set_reuse_frozen(on: bool) -> None:
    """Evaluate the frozen (reference-compatible) RHS once per attempt and
    copy it into the other stages: bit-identical, six times fewer
    transforms for Tsit5."""
    lib().orc_set_reuse_frozen(1 if on else 0)


def set_smooth_convolution(on: bool) -> None:
    """Convolve at the smallest 2/3/5/7-smooth size >= 2n-1 instead of the
    reference's 2n-1 (same linear convolution to rounding, the cost of an
    optimised FFT library); models created afterwards use it."""
    lib().orc_set_smooth_convolution(1 if on else 0)


def set_rhs_noise(eps: float, seed: int = 1) -> None:
    """Add seeded white noise of relative size eps * max|k| to every RHS
    evaluation (a conditioning probe: eps = 1e-7 stands in for the rounding
    of an FP32 right-hand side); 0 turns it off."""
    lib().orc_set_rhs_noise(float(eps), int(seed))


def set_max_rejections(n: int) -> None:
    """Rejected Tsit5 attempts allowed within one update before it fails
    with status 3 (0 restores the default, 1e6)."""
    lib().orc_set_max_rejections(int(n))


def cfft(x: np.ndarray, sign: int = -1) -> np.ndarray:
    re = _f64(np.real(x)).copy()
    im = _f64(np.imag(x)).copy()
    lib().orc_cfft(len(re), _p(re), _p(im), sign)
    return re + 1j * im


def dht2d(a: np.ndarray) -> np.ndarray:
    a = _f64(a)
    out = np.empty_like(a)
    ny, nx = a.shape
    lib().orc_dht2d(nx, ny, _p(a), _p(out))
    return out


def kappa(nx, ny, dx, dy):
    out = np.empty((ny, nx))
    lib().orc_kappa(_p(out), nx, ny, dx, dy)
    return out


def derivative(kind: str, u, d):
    u = _f64(u)
    d = _f64(d)
    out = np.zeros_like(u)
    ny, nx = u.shape
    getattr(lib(), "orc_derivative_" + kind)(_p(out), _p(u), _p(d), nx, ny)
    return out


def lvelva(w, canom_full, mask, g, nu, D, eta, R, kap, dxm, dym, sec_per_year):
    w = _f64(w)
    ny, nx = w.shape
    out = np.empty_like(w)
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    args = [_f64(a) for a in (canom_full, D, eta, R, kap, dxm, dym)]
    lib().orc_lvelva(_p(out), _p(w), _p(args[0]), m.ctypes.data_as(C.POINTER(C.c_uint8)), g, nu,
                     _p(args[1]), _p(args[2]), _p(args[3]), _p(args[4]), nx, ny, _p(args[5]),
                     _p(args[6]), sec_per_year)
    return out


def elastic_green(nx, ny, dx):
    out = np.empty((ny, nx))
    lib().orc_elastic_green(_p(out), nx, ny, dx, dx)
    return out


def zss_green(nx, ny, m_earth, r_earth, dx):
    out = np.empty((ny, nx))
    lib().orc_zss_green(_p(out), nx, ny, m_earth, r_earth, dx, dx)
    return out


def kernel_spectrum(kernel, M):
    kernel = _f64(kernel)
    ny, nx = kernel.shape
    H = M // 2 + 1
    re = np.empty((M, H))
    im = np.empty((M, H))
    lib().orc_kernel_spectrum(nx, ny, M, _p(kernel), _p(re), _p(im))
    return re, im


def conv(spec, inp, M):
    inp = _f64(inp)
    ny, nx = inp.shape
    out = np.empty_like(inp)
    re, im = (_f64(s) for s in spec)
    lib().orc_conv(_p(out), nx, ny, M, _p(re), _p(im), _p(inp))
    return out


def make_params(d: dict) -> OrcParams:
    p = OrcParams()
    for k, v in d.items():
        if k in ("zl", "viscosities"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        elif hasattr(p, k):
            setattr(p, k, v)
    return p


class Model:
    """The oracle's isos_class: create / init_state / update, fields out."""

    def __init__(self, params: dict, nx_ice: int, ny_ice: int, dx: float, dy: float, K=None):
        self.L = lib()
        self.params = make_params(params)
        Kp = None
        self._K = None
        if K is not None:
            self._K = _f64(K)
            Kp = _p(self._K)
        self.h = self.L.orc_create(C.byref(self.params), nx_ice, ny_ice, dx, dy, Kp)
        if not self.h:
            raise ValueError("orc_create rejected the configuration")
        d = (C.c_int32 * 8)()
        self.L.orc_dims(self.h, d)
        self.nx, self.ny, self.icrop1, self.icrop2, self.jcrop1, self.jcrop2 = d[0], d[1], d[2], d[3], d[4], d[5]
        self.nx_ice, self.ny_ice = d[6], d[7]

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fields(self, D_lith=None, eta_eff=None, R=None, maskactive=None):
        D = D_lith
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = _f64(a)
            keep.append(a)
            return _p(a)
        m = None
        if maskactive is not None:
            mm = np.ascontiguousarray(maskactive, dtype=np.uint8)
            keep.append(mm)
            m = mm.ctypes.data_as(C.POINTER(C.c_uint8))
        self.L.orc_set_fields(self.h, ptr(D), ptr(eta_eff), ptr(R), m)

    def init_state(self, z_bed, H_ice, time, bsl: OrcBsl):
        z = _f64(z_bed)
        H = _f64(H_ice)
        return self.L.orc_init_state(self.h, _p(z), _p(H), float(time), C.byref(bsl))

    def update(self, H_ice, time, bsl: OrcBsl):
        H = _f64(H_ice)
        return self.L.orc_update(self.h, _p(H), float(time), C.byref(bsl))

    def field(self, name: str) -> np.ndarray:
        out = np.empty((self.ny, self.nx))
        rc = self.L.orc_get_field(self.h, FIELDS[name], _p(out))
        if rc != 0:
            raise KeyError(name)
        return out

    def crop(self, a: np.ndarray) -> np.ndarray:
        return a[self.jcrop1 - 1:self.jcrop2, self.icrop1 - 1:self.icrop2]

    def scalars(self) -> dict:
        o = np.zeros(16)
        self.L.orc_get_scalars(self.h, _p(o))
        keys = ["t", "dt", "time_diag", "bsl", "V_af", "V_den", "deltaV_bsl", "dbsl_total",
                "n_rhs", "n_accept", "n_reject", "sec_per_year", "cc", "Vden", "M", "bsl_ref"]
        return dict(zip(keys, o.tolist()))

    def rhs_now(self):
        out = np.empty((self.ny, self.nx))
        self.L.orc_rhs_now(self.h, _p(out))
        return out


def make_bsl(method=0, bsl_init=0.0, A_ocean_pd=3.625e14) -> OrcBsl:
    b = OrcBsl()
    b.method = method
    b.constant_ocean_surface = 1
    b.bsl_init = bsl_init
    b.bsl_now = bsl_init
    b.A_ocean_pd = A_ocean_pd
    b.A_ocean_now = A_ocean_pd
    return b


# ---- rheology_file branch of isos_init (src/fastisostasy.f90:262-443) -------

def bilinear_array(xr, yr, z, xo, yo):
    """bilinear_interpolation_array (src/isos_utils.f90:561-575) of z (nyr,
    nxr) at the points xo x yo, in the routine's single precision."""
    xr, yr, z, xo, yo = _f64(xr), _f64(yr), _f64(z), _f64(xo), _f64(yo)
    out = np.zeros((len(yo), len(xo)))
    lib().orc_bilinear_array(_p(xr), len(xr), _p(yr), len(yr), _p(z), _p(xo), len(xo), _p(yo), len(yo), _p(out))
    return out


def smooth_gauss_2d(var, dx, sigma):
    """smooth_gauss_2D (src/isos_utils.f90:696-819); None where the
    reference stops (window wider than the grid)."""
    v = _f64(var).copy()
    if lib().orc_smooth_gauss_2d(_p(v), v.shape[1], v.shape[0], float(dx), float(sigma)):
        return None
    return v


def rheology_file(p: dict, xc, yc, dx, kappa, He, xr, yr, zr=None, thick=None, thick_scale=1.0,
                  log10_eta=None, stddev=None, stddev_scaling=False, radius=0.0, cc=1.0):
    """He, D, eta_eff, R of the padded grid from a rheology file's arrays,
    step by step as isos_init does it: thickness (nyr, nxr), log10 eta and
    stddev (nzr, nyr, nxr).  He: the thickness used without a file
    thickness."""
    ny, nx = len(yc), len(xc)
    n = nx * ny
    He = np.array(He, dtype=np.float64).reshape(ny, nx)
    if thick is not None:
        He = bilinear_array(xr, yr, _f64(thick) * thick_scale, xc, yc)
        if radius > 0:
            He = smooth_gauss_2d(He, dx, radius)
    D = p["E"] * 1e9 * (He * He * He) / (12.0 * (1.0 - p["nu"] * p["nu"]))
    if log10_eta is None:
        return He, D, None, None
    nz = len(zr)
    nl = int(p["nl"])
    depth = np.array([zr[nz - 1] - zr[nz - 1 - q] for q in range(nz)])
    prof = np.stack([bilinear_array(xr, yr, log10_eta[nz - 1 - q], xc, yc) for q in range(nz)])
    if stddev_scaling and stddev is not None:
        sd = np.stack([bilinear_array(xr, yr, stddev[nz - 1 - q], xc, yc) for q in range(nz)])
        prof = prof + p["viscosity_scaling"] * sd
    prof = np.where(prof < 16, 16.0, prof)
    prof = np.where(prof > 23, 23.0, prof)
    bnd = np.zeros((nl, ny, nx))
    bnd[0] = He
    for k in range(1, nl):
        bnd[k] = bnd[k - 1] + p["dl"] if int(p["layering"]) == 1 else p["zl"][k]
    eta3 = np.zeros((nl, ny, nx))
    L = lib()
    dep = _f64(depth)
    col = np.zeros(nz)
    for j in range(ny):
        for i in range(nx):
            col[:] = prof[:, j, i]
            for k in range(nl):
                eta3[k, j, i] = 10.0 ** L.orc_interp_0d(_p(dep), _p(col), nz, float(bnd[k, j, i]))
    eta_eff = np.zeros((ny, nx))
    R = np.zeros((ny, nx))
    e3, b3, kap = _f64(eta3), _f64(bnd), _f64(kappa)
    L.orc_lump3(_p(e3), _p(b3), _p(kap), n, nl, int(p["lumping"]), _p(eta_eff), _p(R))
    if radius > 0:
        eta_eff = smooth_gauss_2d(eta_eff, dx, radius)
    mode = 0 if stddev_scaling else int(p["visc_scaling_method"])
    if mode == 2:
        eta_eff = np.full_like(eta_eff, eta_eff.min())
    elif mode == 3:
        eta_eff = np.full_like(eta_eff, eta_eff.max())
    elif mode == 1:
        eta_eff = eta_eff * p["viscosity_scaling"]
    eta_eff = eta_eff * cc
    eta_eff = np.exp(np.log10(p["eta_ref"] / eta_eff)) * eta_eff
    return He, D, eta_eff, R
