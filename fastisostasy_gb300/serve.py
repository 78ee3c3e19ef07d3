"""Host side of the solve server (fi_serve_* in include/fi_gpu.h).

A request is one independent LV-ELVA solve of a Workload: init at t0 with no
ice (or `H_ref`), then isos_update every `dtt` up to `t_end` under the
workload's final ice load.  The scheduler, admission and device work live in
libfigpu.so; this module only packs requests and unpacks results.
"""
import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from .isostasy import FiError, _f64, make_params

STATE = {0: "queued", 1: "running", 2: "done", 3: "failed"}


def padded_dims(params: dict, nx_ice: int, ny_ice: int, dx: float, dy: Optional[float] = None, precision=0):
    """(nx, ny, icrop1, icrop2, jcrop1, jcrop2) of the padded domain."""
    L = _lib.load()
    out = (C.c_int32 * 6)()
    p = make_params(params, precision)
    rc = L.fi_padded_dims(C.byref(p), int(nx_ice), int(ny_ice), float(dx), float(dx if dy is None else dy), out)
    if rc:
        raise FiError(rc, "fi_padded_dims")
    return tuple(out)


class Server:
    """Continuous-batching server on the current CUDA device."""

    def __init__(self, max_inflight: int = 64, reserve_gb: float = 4.0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.fi_serve_create(int(max_inflight), float(reserve_gb), C.byref(h))
        if rc:
            raise FiError(rc, "fi_serve_create")
        self.h = h
        self._shapes = {}

    def prepare(self, wl, t_end: Optional[float] = None, t0: float = 0.0, precision: int = 0,
                dtt: Optional[float] = None):
        """Pack a Workload into a request (padded fields computed here), so
        that submit_prepared costs only the copy into the server."""
        p = make_params(wl.params, precision)
        nx, ny = padded_dims(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)[:2]
        fields = wl.padded_fields(nx, ny)
        keep = []

        def arr(a, dtype=np.float64):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a

        q = _lib.FiRequest()
        q.p = p
        q.nx_ice, q.ny_ice = wl.nx_ice, wl.ny_ice
        q.dx = q.dy = wl.dx
        zb, H = arr(wl.z_bed), arr(wl.H_final)
        q.z_bed = zb.ctypes.data_as(_lib._dp)
        q.H_ice = H.ctypes.data_as(_lib._dp)
        for name in ("D_lith", "eta_eff", "R"):
            a = arr(fields.get(name))
            if a is not None:
                assert a.shape == (ny, nx), (name, a.shape)
                setattr(q, name, a.ctypes.data_as(_lib._dp))
        m = arr(fields.get("maskactive"), np.uint8)
        if m is not None:
            q.maskactive = m.ctypes.data_as(_lib._u8)
        q.t0 = t0
        q.t_end = wl.t_end if t_end is None else t_end
        q.dtt = wl.dtt if dtt is None else dtt
        q.bsl = 0.0
        return (q, keep, (wl.ny_ice, wl.nx_ice))

    def submit_prepared(self, prep) -> int:
        q, _keep, shape = prep
        rid = C.c_uint64()
        rc = self.L.fi_serve_submit(self.h, C.byref(q), C.byref(rid))   # copies every array
        if rc:
            raise FiError(rc, "fi_serve_submit")
        self._shapes[rid.value] = shape
        return rid.value

    def submit(self, wl, t_end: Optional[float] = None, t0: float = 0.0, precision: int = 0,
               dtt: Optional[float] = None) -> int:
        return self.submit_prepared(self.prepare(wl, t_end, t0, precision, dtt))

    def info(self, rid: int) -> dict:
        i = _lib.FiRequestInfo()
        rc = self.L.fi_serve_info(self.h, C.c_uint64(rid), C.byref(i))
        if rc:
            raise FiError(rc, "fi_serve_info")
        return {"state": STATE[i.state], "status": i.status, "updates": i.updates, "t_submit": i.t_submit,
                "t_admit": i.t_admit, "t_done": i.t_done, "error": i.error.decode(errors="replace")}

    def wait(self, rid: int, timeout: float = 600.0) -> dict:
        i = _lib.FiRequestInfo()
        rc = self.L.fi_serve_wait(self.h, C.c_uint64(rid), float(timeout), C.byref(i))
        if rc:
            raise FiError(rc, "fi_serve_wait")
        return {"state": STATE[i.state], "status": i.status, "updates": i.updates, "t_submit": i.t_submit,
                "t_admit": i.t_admit, "t_done": i.t_done, "error": i.error.decode(errors="replace")}

    def result(self, rid: int):
        """(w, z_bed) on the ice grid; releases the request."""
        shape = self._shapes.pop(rid)
        w = np.empty(shape)
        zb = np.empty(shape)
        rc = self.L.fi_serve_result(self.h, C.c_uint64(rid), w.ctypes.data_as(_lib._dp),
                                    zb.ctypes.data_as(_lib._dp))
        if rc:
            raise FiError(rc, "fi_serve_result")
        return w, zb

    def clock(self) -> float:
        return self.L.fi_serve_clock(self.h)

    def close(self):
        if self.h:
            self.L.fi_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Members (independent domains, any sizes) advanced in lockstep.

    mode "graph": one fi_batch_step per coupling step runs the whole
    ensemble as one CUDA graph whose Tsit5 attempts are batched launches over
    all members (members must run reference-compatible Tsit5).
    mode "streams": fi_batch_update enqueues one isos_update per member on
    the member's own stream (any integrator)."""

    def __init__(self, workloads, precision: int = 1, mode: str = "graph"):
        from .isostasy import Domain
        self.L = _lib.load()
        self.mode = mode
        self.doms = []
        self.bsl = (_lib.FiBsl * len(workloads))()
        for i, wl in enumerate(workloads):
            d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
            f = wl.padded_fields(d.nx, d.ny)
            if f:
                d.set_fields(**f)
            b = self.bsl[i]
            b.method, b.constant_ocean_surface = 0, 1
            b.bsl_init = b.bsl_now = 0.0
            b.A_ocean_pd = b.A_ocean_now = 3.625e14
            d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
            self.doms.append(d)
        self.wls = list(workloads)
        self.hs = (C.c_void_p * len(self.doms))(*[d.h.value for d in self.doms])
        self.batch = None
        if mode == "graph":
            bh = C.c_void_p()
            rc = self.L.fi_batch_create(self.hs, len(self.doms), C.byref(bh))
            if rc:
                raise FiError(rc, "fi_batch_create")
            self.batch = bh
        self.t = 0.0

    def first_update(self, t: float):
        """Apply each member's ice load with a synchronous isos_update."""
        for i, (d, wl) in enumerate(zip(self.doms, self.wls)):
            d.update(wl.H_final, t, self.bsl[i])
        self.t = t

    def update(self, t: float):
        if self.batch is not None:
            rc = self.L.fi_batch_step(self.batch, float(t), self.bsl)
        else:
            rc = self.L.fi_batch_update(self.hs, len(self.doms), float(t), self.bsl)
        if rc:
            raise FiError(rc, "batched update")
        self.t = t

    def synchronize(self):
        st = (C.c_int32 * len(self.doms))()
        if self.batch is not None:
            rc = self.L.fi_batch_wait(self.batch, st)
        else:
            rc = self.L.fi_batch_synchronize(self.hs, len(self.doms), st)
        if rc:
            raise FiError(rc, "ensemble member %d" % next(i for i, v in enumerate(st) if v))

    def close(self):
        if self.batch is not None:
            self.L.fi_batch_destroy(self.batch)
            self.batch = None
        for d in self.doms:
            d.close()
        self.doms = []
