"""Host-side mirror of FastIsostasy's Fortran API for the LV-ELVA path.

Same routine names, argument meaning and error behaviour as module
``fastisostasy`` (src/fastisostasy.f90:33-60) and ``barysealevel``
(src/barysealevel.f90:32-37):

    isos_init(isos, filename, group, nx_ice, ny_ice, dx, dy[, rho_ice][, K])
    isos_init_ref(isos, z_bed, H_ice[, bsl][, dz_ss])
    isos_init_state(isos, z_bed, H_ice, time, bsl)
    isos_update(isos, H_ice, time, bsl)
    isos_end(isos)
    bsl_init(bsl, filename, year_bp);  bsl_update(bsl, year_bp)

The reference stops the program on an error; here every failing call
raises ``FiError`` carrying the C-ABI status.  Arrays are numpy arrays of
shape (ny, nx) in C order, which is the Fortran (nx, ny) column-major layout.
Every computation runs in libfigpu.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from . import params as P
from ._lib import FiBsl, FiError, FiOut, FiParams

OUT_FIELDS = ("z_bed", "z_ss", "dz_ss", "w", "we", "dwdt", "canom_full", "Hice")
OUT_MASKS = ("maskocean", "maskgrounded", "maskcontinent")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def make_params(d: dict, precision: int = 0) -> FiParams:
    p = FiParams()
    for k, v in d.items():
        if k in ("zl", "viscosities"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        elif k in dict(FiParams._fields_):
            setattr(p, k, v)
    p.precision = int(d.get("precision", precision))
    return p


class Domain:
    """One padded LV-ELVA domain on the GPU (an fi_handle)."""

    def __init__(self, params: dict, nx_ice: int, ny_ice: int, dx: float, dy: Optional[float] = None,
                 K: Optional[np.ndarray] = None, precision: int = 0):
        self.L = _lib.load()
        self.params = dict(params)
        self._p = make_params(params, precision)
        self.precision = self._p.precision
        h = C.c_void_p()
        Kp = None
        if K is not None:
            self._K = _f64(K)
            Kp = _dp(self._K)
        rc = self.L.fi_create(C.byref(self._p), int(nx_ice), int(ny_ice), float(dx),
                              float(dx if dy is None else dy), Kp, C.byref(h))
        if rc != 0:
            raise FiError(rc, "fi_create rejected the configuration")
        self.h = h
        d = (C.c_int32 * 8)()
        self.L.fi_dims(self.h, d)
        self.nx, self.ny, self.icrop1, self.icrop2, self.jcrop1, self.jcrop2, self.nx_ice, self.ny_ice = list(d)
        self._H = None

    # -- helpers
    def _check(self, rc):
        if rc != 0:
            msg = self.L.fi_last_error(self.h)
            raise FiError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.L.fi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def crop(self, a):
        return a[self.jcrop1 - 1:self.jcrop2, self.icrop1 - 1:self.icrop2]

    # -- API
    def set_fields(self, D_lith=None, eta_eff=None, R=None, maskactive=None):
        keep = []

        def p(a):
            if a is None:
                return None
            a = _f64(a)
            keep.append(a)
            return _dp(a)
        m = None
        if maskactive is not None:
            mm = np.ascontiguousarray(maskactive, dtype=np.uint8)
            keep.append(mm)
            m = mm.ctypes.data_as(C.POINTER(C.c_uint8))
        self._check(self.L.fi_set_fields(self.h, p(D_lith), p(eta_eff), p(R), m))

    def set_rheology(self, xc, yc, zc=None, litho_thickness=None, litho_thickness_scaling=1.0,
                     log10_viscosity=None, stddev_log10_viscosity=None, stddev_scaling=False,
                     rheo_smoothing_radius=0.0):
        """The rheology_file branches of isos_init from a file's arrays:
        litho_thickness (ny, nx), log10_viscosity / its stddev (nz, ny, nx),
        coordinates ascending (fi_set_rheology)."""
        keep = []

        def p(a):
            if a is None:
                return None
            a = _f64(a)
            keep.append(a)
            return _dp(a)
        r = _lib.FiRheology()
        r.nx, r.ny = len(xc), len(yc)
        r.nz = 0 if zc is None else len(zc)
        r.xc, r.yc, r.zc = p(xc), p(yc), p(zc)
        r.litho_thickness, r.litho_thickness_scaling = p(litho_thickness), float(litho_thickness_scaling)
        r.log10_viscosity, r.stddev_log10_viscosity = p(log10_viscosity), p(stddev_log10_viscosity)
        r.stddev_scaling = 1 if stddev_scaling else 0
        r.rheo_smoothing_radius = float(rheo_smoothing_radius)
        self._check(self.L.fi_set_rheology(self.h, C.byref(r)))

    OUTPUT_FIELDS = ("z_bed", "z_ss", "dz_ss", "w", "we", "dwdt", "canom_full", "Hice",
                     "maskocean", "maskgrounded", "maskcontinent")

    def output_async(self, dst_ptr: int):
        """Snapshot isos%out after the updates enqueued so far and copy it to
        host memory at dst_ptr (output_bytes() bytes) while later updates
        run (fi_output_async)."""
        self._check(self.L.fi_output_async(self.h, C.c_void_p(dst_ptr)))

    def output_wait(self):
        self._check(self.L.fi_output_wait(self.h))

    def output_bytes(self) -> int:
        return int(self.L.fi_output_bytes(self.h))

    def unpack_output(self, buf: np.ndarray) -> dict:
        """The fields of an output snapshot (buf: float64, output_bytes()/8)."""
        a = np.asarray(buf, dtype=np.float64).reshape(11, self.ny_ice, self.nx_ice)
        out = {k: a[i] for i, k in enumerate(self.OUTPUT_FIELDS)}
        for k in ("maskocean", "maskgrounded", "maskcontinent"):
            out[k] = out[k] != 0.0
        return out

    def set_kernels(self, GE=None, GN=None):
        a = _f64(GE) if GE is not None else None
        b = _f64(GN) if GN is not None else None
        self._check(self.L.fi_set_kernels(self.h, _dp(a) if a is not None else None,
                                          _dp(b) if b is not None else None))

    def init_ref(self, z_bed, H_ice, bsl=0.0, dz_ss=None):
        z = _f64(z_bed)
        H = _f64(H_ice)
        d = _f64(dz_ss) if dz_ss is not None else None
        self._check(self.L.fi_init_ref(self.h, _dp(z), _dp(H), float(bsl), _dp(d) if d is not None else None))

    def init_state(self, z_bed, H_ice, time, bsl: FiBsl):
        z = _f64(z_bed)
        H = _f64(H_ice)
        self._check(self.L.fi_init_state(self.h, _dp(z), _dp(H), float(time), C.byref(bsl)))

    def update(self, H_ice, time, bsl: FiBsl, out: Optional[dict] = None):
        H = _f64(H_ice)
        o = None
        if out is not None:
            o = FiOut()
            for k in OUT_FIELDS:
                if k in out:
                    setattr(o, k, _dp(out[k]))
            for k in OUT_MASKS:
                if k in out:
                    setattr(o, k, out[k].ctypes.data_as(C.POINTER(C.c_uint8)))
        rc = self.L.fi_update(self.h, _dp(H), float(time), C.byref(bsl), C.byref(o) if o is not None else None)
        self._check(rc)

    def update_async(self, d_H_ice_ptr, time, bsl: FiBsl):
        self._check(self.L.fi_update_async(self.h, C.c_void_p(d_H_ice_ptr) if d_H_ice_ptr else None,
                                           float(time), C.byref(bsl)))

    def synchronize(self):
        self._check(self.L.fi_synchronize(self.h))

    def field(self, name: str) -> np.ndarray:
        out = np.empty((self.ny, self.nx))
        self._check(self.L.fi_get_field(self.h, _lib.FIELDS[name], _dp(out)))
        return out

    def scalars(self) -> dict:
        o = np.zeros(16)
        self._check(self.L.fi_get_scalars(self.h, _dp(o)))
        keys = ["t", "dt", "time_diag", "bsl", "V_af", "V_den", "deltaV_bsl", "dbsl_total", "n_rhs",
                "n_accept", "n_reject", "sec_per_year", "cc", "Vden", "conv_size", "bsl_ref"]
        return dict(zip(keys, o.tolist()))

    def lvelva(self, w, canom_full):
        w = _f64(w)
        cf = _f64(canom_full)
        out = np.empty_like(w)
        self._check(self.L.fi_lvelva(self.h, _dp(w), _dp(cf), _dp(out)))
        return out

    def convolve(self, kernel: int, x):
        x = _f64(x)
        out = np.empty_like(x)
        self._check(self.L.fi_convolve(self.h, int(kernel), _dp(x), _dp(out)))
        return out

    def metrics(self) -> dict:
        """Run metrics of the handle (fi_metrics_json)."""
        import json
        buf = C.create_string_buffer(1024)
        self._check(self.L.fi_metrics_json(self.h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def state_export(self) -> np.ndarray:
        buf = np.zeros(self.L.fi_state_size(self.h))
        self._check(self.L.fi_state_export(self.h, _dp(buf)))
        return buf

    def state_import(self, buf):
        b = _f64(buf)
        self._check(self.L.fi_state_import(self.h, _dp(b)))


# ---------------------------------------------------------------------------
# The reference's call surface
# ---------------------------------------------------------------------------
class BslClass:
    """bsl_class (src/barysealevel.f90:16-29)."""

    def __init__(self):
        self.c = FiBsl()
        self._keep = []

    @property
    def bsl_now(self):
        return self.c.bsl_now

    @property
    def A_ocean_now(self):
        return self.c.A_ocean_now


def bsl_init(bsl: BslClass, filename: Optional[str] = None, year_bp: float = 0.0, *, method: str = None,
             bsl_init_value: float = None, A_ocean_pd: float = None, series=None, aocean_table=None):
    """bsl_init (src/barysealevel.f90:40-106).  File-based series are passed as
    arrays (`series=(time, value)`, `aocean_table=(bsl, A_ocean)`)."""
    d = {"method": "const", "bsl_init": 0.0, "A_ocean_pd": 3.625e14}
    if filename is not None:
        with open(filename) as fh:
            d.update(P.read_namelist(fh.read(), "barysealevel"))
    if method is not None:
        d["method"] = method
    if bsl_init_value is not None:
        d["bsl_init"] = bsl_init_value
    if A_ocean_pd is not None:
        d["A_ocean_pd"] = A_ocean_pd
    c = bsl.c
    c.method = P.BSL_METHOD[str(d["method"])]
    c.bsl_init = float(d["bsl_init"])
    c.bsl_now = c.bsl_init
    c.A_ocean_pd = float(d["A_ocean_pd"])
    c.A_ocean_now = c.A_ocean_pd
    c.constant_ocean_surface = 1 if aocean_table is None else 0
    if series is not None:
        t, v = (_f64(a) for a in series)
        bsl._keep += [t, v]
        c.series_t, c.series_v, c.n_series = _dp(t), _dp(v), len(t)
    if aocean_table is not None:
        b, a = (_f64(x) for x in aocean_table)
        bsl._keep += [b, a]
        c.bsl_vec, c.aocean_vec, c.n_aocean = _dp(b), _dp(a), len(b)
    bsl_update(bsl, year_bp)


def bsl_update(bsl: BslClass, year_bp: float):
    rc = _lib.load().fi_bsl_update(C.byref(bsl.c), float(year_bp))
    if rc != 0:
        raise FiError(rc, "bsl_update")


class IsosClass:
    """isos_class (src/isostasy_defs.f90:202-209): par, domain, out."""

    def __init__(self):
        self.dom: Optional[Domain] = None
        self.par: dict = {}
        self.out: dict = {}


def isos_init(isos: IsosClass, filename: Optional[str], group: str, nx_ice: int, ny_ice: int, dx: float,
              dy: float, rho_ice: Optional[float] = None, K: Optional[np.ndarray] = None, *,
              params: Optional[dict] = None, precision: int = 0):
    """isos_init (src/fastisostasy.f90:64-473).  `params` (SI units) may be
    given instead of a namelist file."""
    par = dict(params) if params is not None else P.load(filename, group)
    if rho_ice is not None:
        par["rho_ice"] = rho_ice
    isos.par = par
    isos.dom = Domain(par, nx_ice, ny_ice, dx, dy, K=K, precision=precision)
    isos.out = {k: np.zeros((ny_ice, nx_ice)) for k in OUT_FIELDS}
    isos.out.update({k: np.zeros((ny_ice, nx_ice), dtype=np.uint8) for k in OUT_MASKS})


def isos_init_ref(isos: IsosClass, z_bed, H_ice, bsl: Optional[float] = None, dz_ss=None):
    isos.dom.init_ref(z_bed, H_ice, 0.0 if bsl is None else bsl, dz_ss)


def isos_init_state(isos: IsosClass, z_bed, H_ice, time: float, bsl: BslClass):
    isos.dom.init_state(z_bed, H_ice, time, bsl.c)


def isos_update(isos: IsosClass, H_ice, time: float, bsl: BslClass):
    isos.dom.update(H_ice, time, bsl.c, out=isos.out)


def isos_end(isos: IsosClass):
    if isos.dom is not None:
        isos.dom.close()
        isos.dom = None
