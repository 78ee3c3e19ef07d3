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

STATE = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}


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

    def cancel(self, rid: int) -> None:
        """Cancel a queued or running request (fi_serve_cancel)."""
        rc = self.L.fi_serve_cancel(self.h, C.c_uint64(rid))
        if rc:
            raise FiError(rc, "fi_serve_cancel")

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

    mode "graph": one fi_batch_step per coupling step runs a group of
    members as one CUDA graph whose Tsit5 attempts are batched launches over
    the group (members must run reference-compatible Tsit5).  With
    groups > 1 the members are sorted by an estimate of their stiffness
    (max D / (eta dx^3), which sets how many attempts an update needs) and
    split into that many groups, each a batch on its own stream, so a stiff
    member holds back only the members of its own group; with `priority`
    the stiffest group's stream has the device's highest priority; with
    `autotune` each batch's transform and stencil shapes are chosen by
    timing candidates on its own members (fi_batch_autotune).
    mode "streams": fi_batch_update enqueues one isos_update per member on
    the member's own stream (any integrator)."""

    def __init__(self, workloads, precision: int = 1, mode: str = "graph", groups: int = 1,
                 priority: bool = True, autotune: bool = True):
        from .isostasy import Domain
        self.L = _lib.load()
        self.mode = mode
        self.doms = []
        n = len(workloads)
        stiff = []
        for wl in workloads:
            d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
            f = wl.padded_fields(d.nx, d.ny)
            if f:
                d.set_fields(**f)
            self.doms.append(d)
            if mode == "graph" and groups > 1:
                stiff.append(float(np.max(d.field("D_lith") / d.field("eta_eff"))) / wl.dx ** 3)
        order = sorted(range(n), key=lambda i: -stiff[i]) if stiff else list(range(n))
        ng = max(1, min(groups if mode == "graph" else 1, n))
        self.groups = [order[g * n // ng:(g + 1) * n // ng] for g in range(ng)]
        self.slot = {}
        self.bsls = []
        for g, members in enumerate(self.groups):
            arr = (_lib.FiBsl * len(members))()
            for j, i in enumerate(members):
                self.slot[i] = (g, j)
            self.bsls.append(arr)
        for i, (d, wl) in enumerate(zip(self.doms, workloads)):
            b = self.bsl_of(i)
            b.method, b.constant_ocean_surface = 0, 1
            b.bsl_init = b.bsl_now = 0.0
            b.A_ocean_pd = b.A_ocean_now = 3.625e14
            d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        self.wls = list(workloads)
        self.hss = [(C.c_void_p * len(m))(*[self.doms[i].h.value for i in m]) for m in self.groups]
        self.batches = []
        self.shapes = []   # autotuned (rows, columns, strip rows, waves) per batch
        if mode == "graph":
            for g, (hs, m) in enumerate(zip(self.hss, self.groups)):
                bh = C.c_void_p()
                rc = self.L.fi_batch_create(hs, len(m), C.byref(bh))
                if rc:
                    raise FiError(rc, "fi_batch_create")
                self.batches.append(bh)
                if autotune:
                    shape = (C.c_int32 * 4)()
                    rc = self.L.fi_batch_autotune(bh, shape)
                    if rc:
                        raise FiError(rc, "fi_batch_autotune")
                    self.shapes.append(tuple(shape))
                if g == 0 and len(self.groups) > 1 and priority:
                    # the stiffest group has the longest chain of attempts:
                    # its launches go first, the other groups fill idle SMs
                    rc = self.L.fi_batch_set_priority(bh, 1)
                    if rc:
                        raise FiError(rc, "fi_batch_set_priority")
        self.t = 0.0

    def bsl_of(self, i):
        g, j = self.slot[i]
        return self.bsls[g][j]

    def first_update(self, t: float):
        """Apply each member's ice load with a synchronous isos_update."""
        for i, (d, wl) in enumerate(zip(self.doms, self.wls)):
            d.update(wl.H_final, t, self.bsl_of(i))
        self.t = t

    def update(self, t: float):
        for g, m in enumerate(self.groups):
            if self.batches:
                rc = self.L.fi_batch_step(self.batches[g], float(t), self.bsls[g])
            else:
                rc = self.L.fi_batch_update(self.hss[g], len(m), float(t), self.bsls[g])
            if rc:
                raise FiError(rc, "batched update")
        self.t = t

    def synchronize(self):
        for g, m in enumerate(self.groups):
            st = (C.c_int32 * len(m))()
            if self.batches:
                rc = self.L.fi_batch_wait(self.batches[g], st)
            else:
                rc = self.L.fi_batch_synchronize(self.hss[g], len(m), st)
            if rc:
                raise FiError(rc, "ensemble member %d" % m[next(j for j, v in enumerate(st) if v)])

    def close(self):
        for b in self.batches:
            self.L.fi_batch_destroy(b)
        self.batches = []
        for d in self.doms:
            d.close()
        self.doms = []
