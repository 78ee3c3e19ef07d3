"""Shared test helpers: paired GPU / oracle runs of one workload."""
import numpy as np

from fastisostasy_gb300 import _lib
from fastisostasy_gb300 import workloads as W
from fastisostasy_gb300.isostasy import Domain
from oracle import oracle as O


def gpu_bsl(method=0, bsl_init=0.0, A_ocean_pd=3.625e14):
    b = _lib.FiBsl()
    b.method = method
    b.constant_ocean_surface = 1
    b.bsl_init = bsl_init
    b.bsl_now = bsl_init
    b.A_ocean_pd = A_ocean_pd
    b.A_ocean_now = A_ocean_pd
    return b


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


class Pair:
    """Runs the same workload through the GPU library and the oracle."""

    def __init__(self, wl: W.Workload, precision=0, gpu=True):
        self.wl = wl
        self.orc = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        self.dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision) if gpu else None
        f = wl.padded_fields(self.orc.nx, self.orc.ny)
        if f:
            self.orc.set_fields(**f)
            if self.dom is not None:
                self.dom.set_fields(**f)
        m = wl.bsl.get("method", 0)
        self.bo = O.make_bsl(m, wl.bsl.get("bsl_init", 0.0), wl.bsl.get("A_ocean_pd", 3.625e14))
        self.bg = gpu_bsl(m, wl.bsl.get("bsl_init", 0.0), wl.bsl.get("A_ocean_pd", 3.625e14))
        self.t = 0.0

    def init(self, t0=0.0):
        self.t = t0
        rc = self.orc.init_state(self.wl.z_bed, self.wl.H_at(t0), t0, self.bo)
        assert rc == 0
        if self.dom is not None:
            self.dom.init_state(self.wl.z_bed, self.wl.H_at(t0), t0, self.bg)

    def step(self, n=1):
        for _ in range(n):
            self.t += self.wl.dtt
            O.lib().orc_bsl_update(self.bo, self.t)
            rc = self.orc.update(self.wl.H_at(self.t), self.t, self.bo)
            assert rc == 0, "oracle update failed with %d at t=%g" % (rc, self.t)
            if self.dom is not None:
                _lib.load().fi_bsl_update(self.bg, self.t)
                self.dom.update(self.wl.H_at(self.t), self.t, self.bg)

    def close(self):
        if self.dom is not None:
            self.dom.close()
        self.orc.close()


def oracle_solve(wl: W.Workload, times, stage_mode=None, eta_scale=1.0, counts=False, rhs_noise=0.0):
    """w on the padded grid after isos_update at each of `times`, from no
    ice at t = 0 under the workload's final load (the serve / ensemble
    solve), by the oracle on every host core; `eta_scale` multiplies the
    workload's viscosity field and `rhs_noise` adds seeded white noise of
    that size relative to max|k| to every right-hand side (perturbations to
    measure conditioning); with `counts`, also the accepted and rejected
    step counts."""
    import os
    O.set_threads(os.cpu_count() or 1)
    p = dict(wl.params)
    if stage_mode is not None:
        p["stage_mode"] = stage_mode
    m = O.Model(p, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
    f = wl.padded_fields(m.nx, m.ny)
    if eta_scale != 1.0:
        f["eta_eff"] = f["eta_eff"] * eta_scale
    if f:
        m.set_fields(**f)
    b = O.make_bsl()
    m.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
    if rhs_noise:
        O.set_rhs_noise(rhs_noise, 99)
    try:
        for t in times:
            rc = m.update(wl.H_final, t, b)
            assert rc == 0, "oracle update failed with %d at t=%g" % (rc, t)
    finally:
        O.set_rhs_noise(0.0)
    w = m.field("w")
    sc = m.scalars()
    m.close()
    return (w, (sc["n_accept"], sc["n_reject"])) if counts else w


def mixed_bound(wl: W.Workload, times, w_oracle):
    """The mixed form's bound against the FP64 oracle for one solve: 1e-5 of
    max|w|, or ten times the move of the oracle's own solution under white
    noise of FP32 size (1e-7 of max|k|) added to every right-hand side,
    where the solve amplifies such noise.  The reference's Tsit5 (one frozen RHS per
    attempt, i.e. forward-Euler steps sized by an error estimate that does
    not see stability) can step past the stability limit of the stiffest,
    grid-scale modes, where any rounding noise then grows geometrically: the
    FP32 right-hand side starts that noise 1e9 times higher than FP64 does,
    and the FP64 solution itself drifts from the same solve computed in
    another order by the same factor per step."""
    sens = rel(oracle_solve(wl, times, rhs_noise=1e-7), w_oracle)
    return max(1e-5, 10.0 * sens), sens
