#!/usr/bin/env python3
"""LV-ELVA benchmark: simulated kyr/s on a 512 x 512 domain, mixed FP32/FP64
form against the plain FP64 form on the same GPU.

Workload (one "step" = one coupling step, i.e. one isos_update call):
  512 x 512 cells at dx = 11.72 km (6000 km square), lithosphere 150 km minus
  a 100 km Gaussian (sigma 500 km) mapped to rigidity with E = 66 GPa,
  nu = 0.28, uniform eta = 1e21 Pa s, centred 1000 km / 1000 m ice disc,
  elastic and geoid convolutions every step (dt_diagnostics = dtt = 10 yr),
  RK4 with true stages at dt = 1 yr (10 RK4 steps = 40 RHS per coupling
  step; dt = 10 yr diverges on this grid).  Inputs are seeded synthetic
  fields; nothing is read from disk.

`value` times fi_update_async with the ice load already resident on the
device; `e2e` times the public fi_update call with host arrays in
page-locked memory (ice load in, every isos%out field back).  L2 is flushed (256 MiB write) between timed
steps, outside the timed events.  `--impl reference` times the CPU
restatement of the reference (the oracle) on the same workload and
integrator (RK4 with true stages) on all host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "LV-ELVA kyr/s @512² mixed vs FP64, same GPU (err≤1e-5); serve p50/p99 ms"
N_CELLS = 512
DX = 11.71875e3
DT = 1.0
DTT = 10.0
WORKLOAD = ("lvelva_512x512_gaussian_lithosphere_disc_rk4_dt1yr_elastic_geoid "
            "(512^2 at 11.72 km, He 150-100 km Gaussian, eta 1e21, 1000 km/1000 m disc, "
            "RK4 true stages dt=1 yr, coupling dtt=10 yr, elastic+geoid every step)")


def workload(stage_mode=1):
    from fastisostasy_gb300 import workloads as W
    return W.config2(n=N_CELLS, L=N_CELLS * DX, dt=DT, dtt=DTT, stage_mode=stage_mode)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "20"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(kernel, dom, precision, stage_mode, rk_steps=int(round(DTT / DT))):
    """Compulsory bytes one launch of `kernel` must move (inputs read once,
    outputs written once, intermediate FFT passes excluded) on the padded
    domain.  Per cell, with s = 8 state bytes and f field bytes (8 plain, 4
    mixed): one RK4 step with true stages reads the state and the four static
    RHS fields at each of 4 stages, the previous stage output at 3 of them,
    writes 4 stage outputs, and the final combination reads x and k1..k4 and
    writes x: 6s + 27f."""
    f = 4 if precision == 1 else 8
    nx, ny = dom.nx, dom.ny
    n = nx * ny
    spec = ny * (nx // 2 + 1) * 2 * f
    px, py = 2 * nx, 2 * ny
    cspec_in = ny * (px // 2 + 1) * 2 * f
    cspec_k = py * (px // 2 + 1) * 2 * f
    cspec_out = (ny + 2) * (px // 2 + 1) * 2 * f
    # the mixed true-stage kernel sequence reads x as a float pair, the
    # previous stage output (3 stages of 4) and dxw = (x - w_ref) of the
    # pairs; it splits x once per update (rk_stage: x and the w_ref pair in,
    # the x pair and dxw out) and advances the pair and dxw in the final
    # combination
    pairs = precision == 1 and stage_mode == 1
    state = (8 + 3 + 4) if pairs else 8 + (8 if stage_mode == 1 else 0)
    table = {
        "flexure": n * (state + 3 * f + 1 + f),
        "rows_fwd": n * f + spec,
        "cols_hartley": 2 * spec + spec // 2,
        "rows_inv": spec + n * f,
        "conv_rows_fwd": n * f + cspec_in,
        "conv_cols": cspec_in + cspec_k + cspec_out,
        "conv_rows_inv": cspec_out + n * 8,
        "rk_stage": n * (8 + 8 + 12) if pairs else n * (8 + f + 8),
        "rk_final": n * (8 + 4 * f + 16 + (28 if pairs else 0)),
        "engine": n * rk_steps * (6 * 8 + 27 * f) if stage_mode == 1 else None,
    }
    return table.get(kernel)


def update_bytes(dom, precision, rk_steps=int(round(DTT / DT))):
    """Compulsory bytes of one whole coupling step per cell: rk_steps RK4
    true-stage steps (6s + 27f), the elastic + geoid convolutions
    (2 x [in f + kernel spectrum 4f + out f]) and the sea-level / mask pass
    (about 15f + 3)."""
    f = 4 if precision == 1 else 8
    return dom.nx * dom.ny * (rk_steps * (6 * 8 + 27 * f) + 12 * f + 15 * f + 3)


def ncu_value(name, kernel):
    """A figure `name[kernel] = value` of the committed ncu summaries in
    profiles/, or None when no capture of it is committed."""
    import glob
    import re
    pat = re.compile(r"%s\[%s\]\s*=\s*([0-9.eE+]+)" % (re.escape(name), re.escape(kernel)))
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as fh:
            m = pat.search(fh.read())
        if m:
            return float(m.group(1))
    return None


def l2_line(kernel, launch_us):
    """The dominant kernel against the L2 instead of HBM: L2 bytes per launch
    (lts__t_sectors.sum x 32 B) from the committed capture over this run's
    launch time, and the capture's lts__throughput fraction of the L2 peak."""
    b = ncu_value("l2_bytes_per_launch", kernel)
    if not b or not launch_us:
        return None
    return {"bytes_per_launch": b, "achieved_gbs": b / (launch_us * 1e-6) / 1e9,
            "frac_of_l2_peak_ncu": ncu_value("l2_throughput_frac", kernel),
            "source": "lts__t_sectors.sum x 32 B and lts__throughput of the committed ncu capture"}


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` (dram__bytes_read.sum +
    dram__bytes_write.sum) from the committed ncu summaries."""
    return ncu_value("traffic_per_launch", kernel)


def make_domain(precision, stage_mode=1):
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib
    wl = workload(stage_mode)
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
    dom.set_fields(**wl.padded_fields(dom.nx, dom.ny))
    b = _lib.FiBsl()
    b.method, b.constant_ocean_surface, b.bsl_init, b.bsl_now = 0, 1, 0.0, 0.0
    b.A_ocean_pd = b.A_ocean_now = 3.625e14
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
    return dom, wl, b


def output_leg(dom, wl, b, steps, t0):
    """ms per update of device-resident updates with and without an
    asynchronous output snapshot (fi_output_async into page-locked memory)
    after every update; the snapshot's copy overlaps the next update."""
    import torch
    H = torch.from_numpy(np.ascontiguousarray(wl.H_final)).to("cuda")
    buf = torch.empty(dom.output_bytes() // 8, dtype=torch.float64).pin_memory()
    ext = torch.cuda.ExternalStream(dom.L.fi_stream(dom.h))
    t = t0
    res = {}
    for with_out in (False, True):
        for _ in range(2):   # warm-up
            t += wl.dtt
            dom.update_async(H.data_ptr(), t, b)
            if with_out:
                dom.output_async(buf.data_ptr())
        dom.output_wait()
        dom.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(steps):
            t += wl.dtt
            dom.update_async(H.data_ptr(), t, b)
            if with_out:
                dom.output_async(buf.data_ptr())
        dom.output_wait()
        e1.record(ext)
        dom.synchronize()
        res["with" if with_out else "without"] = e0.elapsed_time(e1) / steps
    return {"ms_per_step_without": res["without"], "ms_per_step_with": res["with"],
            "bytes_per_snapshot": dom.output_bytes(),
            "note": "e1 is recorded after fi_output_wait, so the last copy is inside the timed region"}


def run_resident(dom, wl, b, steps, warmup, flush, t0=0.0, sampler_index=None, profile=False):
    """Device-resident loop from model time t0: returns (per-step ms list,
    launches, clocks, per-kernel profile, final time)."""
    import torch
    ext = torch.cuda.ExternalStream(dom.L.fi_stream(dom.h))
    H = torch.from_numpy(np.ascontiguousarray(wl.H_final)).to("cuda")
    t = t0
    for _ in range(warmup):
        t += wl.dtt
        dom.update_async(H.data_ptr(), t, b)
    dom.synchronize()
    if profile:
        dom.L.fi_profile(dom.h, -1)
        dom.L.fi_profile(dom.h, 1)
    l0 = dom.L.fi_launch_count(dom.h)
    sampler = ClockSampler(sampler_index) if sampler_index is not None else None
    evs = []
    for _ in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
        t += wl.dtt
        dom.update_async(H.data_ptr(), t, b)
        e1.record(ext)
        evs.append((e0, e1))
    dom.synchronize()
    clocks = sampler.stop() if sampler is not None else None
    launches = dom.L.fi_launch_count(dom.h) - l0
    ms = [a.elapsed_time(c) for a, c in evs]
    prof = None
    if profile:
        import ctypes as C
        from fastisostasy_gb300 import _lib
        nk = len(_lib.PROFILE_KERNELS)
        tot = (C.c_double * nk)()
        cnt = (C.c_longlong * nk)()
        dom.L.fi_profile_read(dom.h, tot, cnt, nk)
        dom.L.fi_profile(dom.h, 0)
        prof = {k: (tot[i], cnt[i]) for i, k in enumerate(_lib.PROFILE_KERNELS) if cnt[i] > 0}
    return ms, launches, clocks, prof, t


def run_e2e(dom, wl, b, steps, warmup, flush, t0):
    """fi_update with host arrays in page-locked memory (the ice load in,
    every output field and mask out), which the call copies to and from the
    device directly."""
    import torch
    ni = (wl.ny_ice, wl.nx_ice)

    def pinned(dtype):
        return torch.zeros(ni, dtype=dtype, pin_memory=True).numpy()

    out = {k: pinned(torch.float64) for k in ("z_bed", "z_ss", "dz_ss", "w", "we", "dwdt", "canom_full", "Hice")}
    out.update({k: pinned(torch.uint8) for k in ("maskocean", "maskgrounded", "maskcontinent")})
    H = pinned(torch.float64)
    H[...] = wl.H_final
    t = t0
    for _ in range(warmup):
        t += wl.dtt
        dom.update(H, t, b, out=out)
    secs = 0.0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t += wl.dtt
        a = time.perf_counter()
        dom.update(H, t, b, out=out)
        secs += time.perf_counter() - a
    h2d = H.nbytes
    # outputs travel as 8 double fields and 3 byte masks (ice grids above
    # 65536 cells; smaller ones as 11 packed doubles)
    d2h = (8 * 8 + 3) * H.size if H.size >= (1 << 16) else 11 * H.size * 8
    return secs, h2d, d2h


def cpu_model():
    """The host CPU's model name and core count (lscpu, else /proc/cpuinfo)."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                name = line.split(":", 1)[1].strip()
                break
        if name is None:
            for line in out.splitlines():
                if line.lower().startswith("vendor id"):
                    name = line.split(":", 1)[1].strip()
    except Exception:
        pass
    if name is None:
        try:
            with open("/proc/cpuinfo") as fh:
                for line in fh:
                    if line.lower().startswith(("model name", "cpu part")):
                        name = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    import platform
    return {"model": name or "unknown", "arch": platform.machine(), "host_cores": os.cpu_count()}


def cpu_baseline(samples=8, threads=1, stage_mode=1):
    """The oracle (C restatement) on the same workload, `samples` coupling
    steps, convolving at the smallest 2/3/5/7-smooth size >= 2n-1 (1024 for
    the reference's 1023 = 3*11*31: the same linear convolution at the cost
    of an optimised FFT library, where this file's FFT would evaluate the
    radix-11 and radix-31 stages as direct sums)."""
    from oracle import oracle as O
    O.set_threads(threads)
    O.set_smooth_convolution(True)
    wl = workload(stage_mode)
    m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
    m.set_fields(**wl.padded_fields(m.nx, m.ny))
    bo = O.make_bsl()
    m.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bo)
    t = 0.0
    t += wl.dtt
    m.update(wl.H_final, t, bo)   # untimed first step
    a = time.perf_counter()
    for _ in range(samples):
        t += wl.dtt
        rc = m.update(wl.H_final, t, bo)
        if rc:
            raise RuntimeError("oracle update failed %d" % rc)
    secs = time.perf_counter() - a
    m.close()
    O.set_smooth_convolution(False)
    return samples * wl.dtt / 1000.0 / secs, secs


def oracle_leg(headline_updates=3):
    """err_vs_oracle: both GPU forms against the FP64 oracle (all host
    cores) from the same start, on the headline workload (512^2, RK4 true
    stages, `headline_updates` coupling steps) and on configuration 3
    (512 x 1024, interactive sea level, reference-compatible Tsit5, one
    coupling step of a few hundred attempts).  max and RMS of |u_gpu -
    u_oracle| / max|u_oracle| for the displacement w, and the count of mask
    cells that differ."""
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    O.set_reuse_frozen(True)   # bit-identical: the frozen RHS evaluated once per attempt
    masks = ("maskocean", "maskgrounded", "maskcontinent")

    def run(wl, n_up):
        o = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        f = wl.padded_fields(o.nx, o.ny)
        if f:
            o.set_fields(**f)
        bo = O.make_bsl()
        o.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bo)
        a = time.perf_counter()
        t = 0.0
        for _ in range(n_up):
            t += wl.dtt
            rc = o.update(wl.H_at(t), t, bo)
            if rc:
                raise RuntimeError("oracle update failed %d" % rc)
        o_secs = time.perf_counter() - a
        ref = {k: o.field(k) for k in ("w",) + masks}
        sc_o = o.scalars()
        o.close()
        out = {"oracle_s": o_secs, "updates": n_up}
        for prec, key in ((0, "fp64"), (1, "mixed")):
            d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=prec)
            if f:
                d.set_fields(**f)
            b = _lib.FiBsl()
            b.method, b.constant_ocean_surface = 0, 1
            b.A_ocean_pd = b.A_ocean_now = 3.625e14
            d.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
            t = 0.0
            for _ in range(n_up):
                t += wl.dtt
                d.update(wl.H_at(t), t, b)
            w = d.field("w")
            sc = d.scalars()
            wmax = max(np.abs(ref["w"]).max(), 1e-300)
            out[key] = {"max_rel": float(np.abs(w - ref["w"]).max() / wmax),
                        "rms_rel": float(np.sqrt(np.mean((w - ref["w"]) ** 2)) / wmax),
                        "mask_mismatch": int(sum(np.sum(d.field(m) != ref[m]) for m in masks)),
                        "same_step_sequence": bool(sc["n_accept"] == sc_o["n_accept"]
                                                   and sc["n_reject"] == sc_o["n_reject"])}
            d.close()
        out["attempts"] = {"accept": sc_o["n_accept"], "reject": sc_o["n_reject"]}
        return out

    try:
        res = {"headline": run(workload(1), headline_updates), "config3": run(W.config3(), 1)}
    finally:
        O.set_reuse_frozen(False)
    res["note"] = ("FP64 oracle on %d host threads; w after the stated coupling steps from the same start"
                   % (os.cpu_count() or 1))
    return res


def ensemble_leg(n_members=256, n_updates=10):
    """256-member ensemble, mixed form, batched: members sorted by stiffness
    into 2 groups, each one CUDA graph per coupling step whose Tsit5 attempts
    are single launches over the group's members (fi_batch_step), against the same members solved one after another in
    the plain FP64 form; the per-member-stream variant (fi_batch_update) is
    reported beside it.  Each member runs reference-compatible Tsit5 (the
    reference's integrator) from t = 30 yr for n_updates coupling steps of
    10 yr after three untimed ones (load switch-on, first update of its kind,
    graph capture).  Handle set-up is timed separately."""
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300.serve import Ensemble
    from fastisostasy_gb300 import _lib
    wls = [W.ensemble_member(i, stage_mode=0) for i in range(n_members)]
    timed = {}
    for mode in ("graph", "streams"):
        a = time.perf_counter()
        ens = Ensemble(wls, precision=1, mode=mode, groups=2 if mode == "graph" else 1)
        init_s = time.perf_counter() - a
        if mode == "graph":
            shapes = list(ens.shapes)
        ens.first_update(10.0)
        ens.update(20.0)
        ens.update(30.0)   # the first batched update of a kind is captured
        ens.synchronize()
        torch.cuda.synchronize()
        a = time.perf_counter()
        for k in range(n_updates):
            ens.update(40.0 + 10.0 * k)
        ens.synchronize()
        timed[mode] = (time.perf_counter() - a, init_s)
        if mode == "graph":
            w_mixed = [d.field("w") for d in ens.doms]
        ens.close()
    batched_s, init_s = timed["graph"]
    seq_s, seq_init = 0.0, 0.0
    sizes = {}
    w64 = []
    for wl in wls:
        sizes[wl.nx_ice] = sizes.get(wl.nx_ice, 0) + 1
        a = time.perf_counter()
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=0)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        seq_init += time.perf_counter() - a
        d.update(wl.H_final, 10.0, b)
        d.update(wl.H_final, 20.0, b)
        d.update(wl.H_final, 30.0, b)
        a = time.perf_counter()
        for k in range(n_updates):
            d.update(wl.H_final, 40.0 + 10.0 * k, b)
        seq_s += time.perf_counter() - a
        w64.append(d.field("w"))
        d.close()
    mkyr = n_members * n_updates * 10.0 / 1000.0
    # per-member error of the batched mixed run against the same member in FP64
    errs = np.array([float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) for a, b in zip(w_mixed, w64)])
    off = [i for i in range(n_members) if errs[i] > 1e-5]
    # conditioning of those members under the reference's integrator, for a
    # bounded sample of the smaller ones: the FP64 oracle's own move when
    # white noise of FP32 size (1e-7 of max|k|) is added to every right-hand
    # side, a stand-in for the rounding of the mixed form's FP32 RHS, which
    # the stiff modes amplify where accepted steps pass their stability limit
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    O.set_reuse_frozen(True)
    times = [10.0, 20.0, 30.0] + [40.0 + 10.0 * k for k in range(n_updates)]

    def oracle_w(wl, noise):
        m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        f = wl.padded_fields(m.nx, m.ny)
        if f:
            m.set_fields(**f)
        bo = O.make_bsl()
        m.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, bo)
        O.set_rhs_noise(noise, 99)
        try:
            for t in times:
                if m.update(wl.H_final, t, bo):
                    return None
        finally:
            O.set_rhs_noise(0.0)
        w = m.field("w")
        m.close()
        return w

    cond = []
    for i in [i for i in off if wls[i].nx_ice <= 256][:6]:
        wl = wls[i]
        w0, w1 = oracle_w(wl, 0.0), oracle_w(wl, 1e-7)
        if w0 is None or w1 is None:
            continue
        wmax = max(np.abs(w0).max(), 1e-300)
        cond.append({"member": i, "n": wl.nx_ice, "mixed_vs_fp64": float(errs[i]),
                     "fp64_gpu_vs_oracle": float(np.abs(w64[i] - w0).max() / wmax),
                     "oracle_rhs_noise_1e-7_vs_oracle": float(np.abs(w1 - w0).max() / wmax)})
    O.set_reuse_frozen(False)
    # one member over the stated 10 kyr horizon (1000 coupling steps), alone
    # in each form: the smallest grid, so that the horizon fits the run
    hm = min(range(n_members), key=lambda i: (wls[i].nx_ice, i))
    horizon = {}
    for prec, key in ((1, "mixed"), (0, "fp64")):
        wl = wls[hm]
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=prec)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        d.update(wl.H_final, 10.0, b)
        a = time.perf_counter()
        for k in range(2, 1001):
            d.update_async(0, 10.0 * k, b)
        d.synchronize()
        secs = time.perf_counter() - a
        sc = d.scalars()
        horizon[key] = {"kyr_s": 9.99 / secs, "t_end_yr": sc["t"], "accepted": sc["n_accept"],
                        "rejected": sc["n_reject"], "w": d.field("w")}
        d.close()
    wm, wd = horizon["mixed"].pop("w"), horizon["fp64"].pop("w")
    horizon.update({"member": hm, "n": wls[hm].nx_ice, "horizon_kyr": 10.0,
                    "err_mixed_vs_fp64": float(np.abs(wm - wd).max() / max(np.abs(wd).max(), 1e-300))})
    return {
        "horizon_member": horizon,
        "workload": "ensemble: %d members, n in {128,192,256,384,512} (%s), dx 10-30 km, log10 eta Gaussian random "
                    "field (mean 21, std 0.5, 500 km), He 50-150 km, disc 300-1200 km / 500-3000 m; "
                    "reference-compatible Tsit5; %d coupling steps of 10 yr per member (the 10 kyr horizon "
                    "cut to a bounded sample)" % (n_members, sizes, n_updates),
        "unit": "member-kyr/s", "batched_mixed": mkyr / batched_s, "sequential_fp64": mkyr / seq_s,
        "speedup": seq_s / batched_s, "batched_s": batched_s, "sequential_s": seq_s,
        "streams_mixed": mkyr / timed["streams"][0],
        "setup_s": {"batched_mixed": init_s, "sequential_fp64": seq_init},
        "autotuned_shapes": [{"rows_per_block": a_[0], "columns_per_block": a_[1], "strip_rows": a_[2],
                              "waves": a_[3]} for a_ in shapes],
        "err_vs_fp64": {
            "max_rel": float(errs.max()), "median_rel": float(np.median(errs)),
            "rms_rel": float(np.sqrt(np.mean(errs ** 2))),
            "members_within_1e-5": int(n_members - len(off)),
            "outside_sizes": {str(n): sum(1 for i in off if wls[i].nx_ice == n) for n in sorted(sizes)},
            "conditioning_sample": cond,
            "note": "max |w_mixed - w_fp64| / max |w_fp64| per member after the timed steps.  The reference's "
                    "Tsit5 takes one RHS per attempt (a forward-Euler step whose error estimate 0.2 dt |k| "
                    "does not see stability); where its accepted steps pass the stability limit of the "
                    "stiffest, grid-scale modes, rounding noise in them grows geometrically.  The FP32 RHS "
                    "starts that noise 1e9 times higher than FP64: conditioning_sample gives, per member, the "
                    "FP64 oracle's own move under white noise of FP32 size added to every RHS, beside the "
                    "GPU FP64 form's distance from the oracle",
        },
    }


def _fp64_solve(wl, n):
    """One request solved alone in the plain FP64 form: handle set-up, then
    isos_update every dtt to t_end (the served solve's sequence)."""
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib
    d = Domain(wl.params, n, n, wl.dx, precision=0)
    f = wl.padded_fields(d.nx, d.ny)
    if f:
        d.set_fields(**f)
    b = _lib.FiBsl()
    b.method, b.constant_ocean_surface = 0, 1
    b.A_ocean_pd = b.A_ocean_now = 3.625e14
    d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
    t = 0.0
    while t < wl.t_end:
        t = min(t + wl.dtt, wl.t_end)
        d.update(wl.H_final, t, b)
    w = d.crop(d.field("w"))
    d.close()
    return w


def _sequential_fp64(wls, arrivals):
    """A single FIFO worker that solves each request in FP64 as it arrives
    (real time): latency = completion - arrival."""
    t0 = time.perf_counter()
    lat = []
    for wl, a in zip(wls, arrivals):
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        _fp64_solve(wl, wl.nx_ice)
        lat.append(time.perf_counter() - t0 - a)
    span = time.perf_counter() - t0 - arrivals[0]
    lat = np.array(lat) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "throughput_req_per_s": len(wls) / span}


def ensemble_full_leg(n_members=256, horizon=10e3, n_seq=8):
    """Configuration 4 at its stated extent: every member of the 256-member
    ensemble (reference-compatible Tsit5, mixed form, batched graphs in two
    stiffness groups) integrated to 10 kyr from no ice, handle set-up
    excluded; beside it a sample of n_seq members (every 256/n_seq-th)
    solved one after another in FP64 to the same horizon, with their
    difference from the batched mixed result at the end.  The sequential
    time of the whole ensemble is estimated from the sample (labelled as
    such)."""
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300.serve import Ensemble
    from fastisostasy_gb300 import _lib
    wls = [W.ensemble_member(i, stage_mode=0) for i in range(n_members)]
    ens = Ensemble(wls, precision=1, mode="graph", groups=2)
    torch.cuda.synchronize()
    n = int(round(horizon / 10.0))
    a = time.perf_counter()
    err = None
    try:
        ens.first_update(10.0)
        for k in range(2, n + 1):
            ens.update(10.0 * k)
        ens.synchronize()
    except Exception as exc:   # a member that fails its update: reported, not raised
        err = str(exc)
    batched_s = time.perf_counter() - a
    w_mixed = [d.field("w") for d in ens.doms]
    sc = [d.scalars() for d in ens.doms]
    ens.close()
    idx = list(range(0, n_members, max(1, n_members // n_seq)))[:n_seq]
    seq = []
    for i in idx:
        wl = wls[i]
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=0)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        a = time.perf_counter()
        for k in range(1, n + 1):
            d.update(wl.H_final, 10.0 * k, b)
        secs = time.perf_counter() - a
        w64 = d.field("w")
        s64 = d.scalars()
        d.close()
        seq.append({"member": i, "n": wl.nx_ice, "fp64_s": secs,
                    "err_mixed_vs_fp64": float(np.abs(w_mixed[i] - w64).max() / max(np.abs(w64).max(), 1e-300)),
                    "attempts_fp64": s64["n_accept"] + s64["n_reject"],
                    "attempts_mixed": sc[i]["n_accept"] + sc[i]["n_reject"]})
    seq_est = sum(r["fp64_s"] for r in seq) * n_members / len(seq)
    mkyr = n_members * horizon / 1000.0
    return {"workload": "configuration 4 at its stated extent: %d members, reference-compatible Tsit5, mixed, "
                        "batched graphs in 2 stiffness groups, 10 kyr each from no ice" % n_members,
            "unit": "member-kyr/s", "batched_s": batched_s, "batched_mixed": mkyr / batched_s,
            "t_end_yr": sc[0]["t"] if sc else None, "error": err,
            "attempts": {"mean": float(np.mean([x["n_accept"] + x["n_reject"] for x in sc])),
                         "max": float(np.max([x["n_accept"] + x["n_reject"] for x in sc]))},
            "sequential_fp64_sample": seq,
            "sequential_fp64_estimate_s": seq_est, "speedup_estimate": seq_est / batched_s}


def ensemble_true_leg(n_members=64, n_updates=4, groups=2, mode="graph"):
    """Configuration 4's members in Tsit5 with true stages (Dormand-Prince
    5(4) with FSAL, the RHS at every stage state; no reference counterpart)
    as one batched graph per coupling step, mixed form, against the same
    members solved one after another in FP64: member-kyr/s, speed-up and the
    per-member difference.  Members start at t = 30 yr after three untimed
    updates, then n_updates coupling steps of 10 yr are timed."""
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300.serve import Ensemble
    from fastisostasy_gb300 import _lib
    wls = [W.ensemble_member(i, stage_mode=1) for i in range(n_members)]
    ens = Ensemble(wls, precision=1, mode=mode, groups=groups if mode == "graph" else 1)
    ens.first_update(10.0)
    ens.update(20.0)
    ens.update(30.0)
    ens.synchronize()
    torch.cuda.synchronize()
    a = time.perf_counter()
    for k in range(n_updates):
        ens.update(40.0 + 10.0 * k)
    ens.synchronize()
    batched_s = time.perf_counter() - a
    w_mixed = [d.field("w") for d in ens.doms]
    attempts = [d.scalars()["n_accept"] + d.scalars()["n_reject"] for d in ens.doms]
    ens.close()
    seq_s, w64 = 0.0, []
    for wl in wls:
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=0)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        for t in (10.0, 20.0, 30.0):
            d.update(wl.H_final, t, b)
        a = time.perf_counter()
        for k in range(n_updates):
            d.update(wl.H_final, 40.0 + 10.0 * k, b)
        seq_s += time.perf_counter() - a
        w64.append(d.field("w"))
        d.close()
    errs = np.array([float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)) for x, y in zip(w_mixed, w64)])
    mkyr = n_members * n_updates * 10.0 / 1000.0
    return {"workload": "%d ensemble members (configuration 4 draws), Tsit5 with true stages, mixed, %s, "
                        "%d coupling steps of 10 yr after three untimed"
                        % (n_members, "batched graphs in %d stiffness groups" % groups if mode == "graph"
                           else "per-member streams", n_updates),
            "unit": "member-kyr/s", "batched_mixed": mkyr / batched_s, "sequential_fp64": mkyr / seq_s,
            "speedup": seq_s / batched_s, "attempts_per_member": {"mean": float(np.mean(attempts)),
                                                                  "max": float(np.max(attempts))},
            "err_vs_fp64": {"members_within_1e-5": int(np.sum(errs <= 1e-5)), "median_rel": float(np.median(errs)),
                            "max_rel": float(errs.max())}}


def serve_leg(lams=(10, 30, 100, 300, 1000, 2000), n_req=48, reserve_gb=8.0, n_long=6):
    """Continuous batching (configuration 5): Poisson arrivals at rate lam of
    n_req solve requests whose sizes 64^2..1024^2 come in the weights
    0.3/0.3/0.2/0.15/0.05 by quota (so a stream of 48 holds three 1024^2
    requests), random-field rheology, disc or dome load, horizon
    log-uniform 1-100 kyr scaled by 1/100, mixed form, through the solve
    server; latency = completion - submission on the server clock.  Beside
    each rate, the same arrivals served by one FIFO worker that solves every
    request in the plain FP64 form as it arrives, actually run.  A second
    stream of n_long requests (64^2..256^2) keeps the unscaled 1-100 kyr
    horizons: served together, against the same requests solved one after
    another in FP64, with each served result's difference from its FP64
    solve."""
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.serve import Server
    sizes = W.serve_sizes(n_req)
    wls = [W.serve_request(i, n=sizes[i]) for i in range(n_req)]
    srv = Server(max_inflight=64, reserve_gb=reserve_gb)
    preps = [srv.prepare(wl, precision=1) for wl in wls]
    # warm-up: one short request per size (kernel attributes, first captures)
    seen = {}
    for wl in wls:
        if wl.nx_ice not in seen:
            seen[wl.nx_ice] = srv.submit(wl, t_end=30.0, precision=1)
    for rid in seen.values():
        srv.wait(rid, 300.0)
        srv.result(rid)
    rng = np.random.default_rng(12345)
    levels = []
    for lam in lams:
        arr = np.cumsum(rng.exponential(1.0 / lam, n_req))
        t_base = srv.clock() + 0.005
        ids = []
        for k, prep in enumerate(preps):
            while srv.clock() < t_base + arr[k]:
                pass
            ids.append(srv.submit_prepared(prep))
        infos = [srv.wait(i, 600.0) for i in ids]
        for i in ids:
            srv.result(i)
        bad = [f for f in infos if f["state"] != "done"]
        if bad:
            raise RuntimeError("serve: %d requests failed: %s" % (len(bad), bad[0]))
        lat = np.array([f["t_done"] - f["t_submit"] for f in infos]) * 1e3
        span = max(f["t_done"] for f in infos) - min(f["t_submit"] for f in infos)
        levels.append({"lambda_per_s": lam, "p50_ms": float(np.percentile(lat, 50)),
                       "p99_ms": float(np.percentile(lat, 99)), "throughput_req_per_s": n_req / span,
                       "arrivals": arr})
    # the unscaled-horizon stream, served together (a burst)
    long_sizes = [64, 128, 256, 64, 128, 256][:n_long]
    lwls = [W.serve_request(1000 + i, horizon_scale=1.0, n=long_sizes[i]) for i in range(n_long)]
    t0 = srv.clock()
    lids = [srv.submit(wl, precision=1) for wl in lwls]
    linfo = [srv.wait(i, 1200.0) for i in lids]
    lres = [srv.result(i)[0] for i in lids]
    served_span = max(f["t_done"] for f in linfo) - t0
    srv.close()
    # sequential plain FP64, actually run: the same arrivals, one FIFO worker
    for lv in levels:
        arr = lv.pop("arrivals")
        lv["sequential_fp64"] = _sequential_fp64(wls, arr - arr[0])
    a = time.perf_counter()
    lerr = []
    for wl, w32 in zip(lwls, lres):
        w64 = _fp64_solve(wl, wl.nx_ice)
        lerr.append(float(np.abs(w32 - w64).max() / max(np.abs(w64).max(), 1e-300)))
    seq_span = time.perf_counter() - a
    count = {n: sizes.count(n) for n in sorted(set(sizes))}
    return {"workload": "serve stream: %d requests per rate, sizes %s by quota, mixed form, RK4 true stages dt=1 yr, "
                        "coupling 10 yr, horizon log-uniform 1-100 kyr x 1/100 (mean %.0f yr)"
                        % (n_req, count, float(np.mean([w.t_end for w in wls]))),
            "levels": levels,
            "unscaled_horizons": {
                "requests": [{"n": wl.nx_ice, "horizon_yr": wl.t_end, "latency_ms": 1e3 * (f["t_done"] - f["t_submit"]),
                              "err_mixed_vs_fp64": e} for wl, f, e in zip(lwls, linfo, lerr)],
                "served_together_s": served_span, "sequential_fp64_s": seq_span,
                "speedup": seq_span / served_span}}


def scale_leg(sizes=(1024, 2048), n_updates=4):
    """The headline workload (Gaussian lithosphere, disc, RK4 true stages,
    dt = 1 yr, coupling 10 yr, elastic + geoid) on larger grids, where the
    fields no longer fit the 129 MB L2: kyr/s and cell-steps/s of both forms,
    the mixed form's per-kernel CUDA-event profile and the algorithmic GB/s
    of each kernel against the measured HBM peak.  (At 2048^2 the step
    engine's phase-A tiles exceed shared memory and the mixed form runs the
    kernel sequence.)"""
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib
    peak, peak_kind = peaks()
    out = {}
    for n in sizes:
        wl = W.config2(n=n, L=n * DX, dt=DT, dtt=DTT, stage_mode=1)
        res = {}
        for prec in (0, 1):
            d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=prec)
            d.set_fields(**wl.padded_fields(d.nx, d.ny))
            b = _lib.FiBsl()
            b.method, b.constant_ocean_surface, b.bsl_init, b.bsl_now = 0, 1, 0.0, 0.0
            b.A_ocean_pd = b.A_ocean_now = 3.625e14
            d.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
            H = torch.from_numpy(np.ascontiguousarray(wl.H_final)).to("cuda")
            ext = torch.cuda.ExternalStream(d.L.fi_stream(d.h))
            t = 0.0
            for _ in range(2):
                t += wl.dtt
                d.update_async(H.data_ptr(), t, b)
            d.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            for _ in range(n_updates):
                t += wl.dtt
                d.update_async(H.data_ptr(), t, b)
            e1.record(ext)
            d.synchronize()
            ms = e0.elapsed_time(e1) / n_updates
            entry = {"ms_per_update": ms, "kyr_s": DTT / 1000.0 / (ms / 1000.0),
                     "cell_steps_per_s": d.nx * d.ny * (DTT / DT) / (ms / 1000.0)}
            if prec == 1:
                d.L.fi_profile(d.h, -1)
                d.L.fi_profile(d.h, 1)
                for _ in range(n_updates):
                    t += wl.dtt
                    d.update_async(H.data_ptr(), t, b)
                d.synchronize()
                import ctypes as C
                nk = len(_lib.PROFILE_KERNELS)
                msv = (C.c_double * nk)()
                cnt = (C.c_longlong * nk)()
                d.L.fi_profile_read(d.h, msv, cnt, nk)
                d.L.fi_profile(d.h, 0)
                kern = {}
                tot = sum(msv[i] for i in range(nk))
                for i, name in enumerate(_lib.PROFILE_KERNELS):
                    if cnt[i] == 0:
                        continue
                    alg = algorithmic_bytes(name, d, 1, 1)
                    us = 1000.0 * msv[i] / cnt[i]
                    gbs = alg / (us * 1e-6) / 1e9 if alg else None
                    kern[name] = {"share": round(msv[i] / tot, 4), "avg_launch_us": round(us, 2),
                                  "alg_GBs": round(gbs, 1) if gbs else None,
                                  "frac_of_peak": round(gbs / peak, 3) if gbs else None}
                entry["kernels"] = kern
                entry["step_engine"] = "engine" in kern
            res["fp64" if prec == 0 else "mixed"] = entry
            d.close()
        res["mixed_over_fp64"] = res["fp64"]["ms_per_update"] / res["mixed"]["ms_per_update"]
        out["%dx%d" % (n, n)] = res
    out["peak"] = {"value": peak, "unit": "GB/s", "kind": peak_kind}
    return out


def engine_trace_leg(n=512):
    """Phase timestamps of the step engine (fi_engine_trace: block 0 stamps
    %globaltimer at every phase and sub-phase boundary of the first RK4 step
    of an update) on the headline workload at n^2, from an eager-launch
    handle (a captured graph keeps the trace setting it was captured with).
    Returns the intervals in microseconds."""
    import ctypes as C
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib
    prev = os.environ.get("FI_NO_GRAPHS")
    os.environ["FI_NO_GRAPHS"] = "1"
    try:
        wl = W.config2(n=n, L=n * DX, dt=DT, dtt=DTT, stage_mode=1)
        d = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
    finally:
        if prev is None:
            del os.environ["FI_NO_GRAPHS"]
        else:
            os.environ["FI_NO_GRAPHS"] = prev
    d.set_fields(**wl.padded_fields(d.nx, d.ny))
    b = _lib.FiBsl()
    b.method, b.constant_ocean_surface = 0, 1
    b.A_ocean_pd = b.A_ocean_now = 3.625e14
    d.init_state(wl.z_bed, wl.H_at(0.0), 0.0, b)
    buf = (C.c_ulonglong * 256)()
    d.L.fi_engine_trace(d.h, buf, 256)
    H = torch.from_numpy(np.ascontiguousarray(wl.H_final)).to("cuda")
    for t in (10.0, 20.0, 30.0, 40.0):
        d.update_async(H.data_ptr(), t, b)
    d.synchronize()
    d.L.fi_engine_trace(d.h, buf, 256)
    d.close()
    ts = [v for v in buf if v]
    return {"n": n, "intervals_us": [round((ts[i + 1] - ts[i]) / 1000.0, 2) for i in range(len(ts) - 1)]}


def configs_leg():
    """The other configurations as bounded samples: config 1 (128^2 uniform
    disc, reference-compatible Tsit5), config 2 (256^2 Gaussian lithosphere,
    RK4 true stages dt = 1 yr) and config 3 (336 x 560 ice grid padded to
    512 x 1024, interactive sea level, two-layer freqdomain mantle,
    reference-compatible Tsit5).  Each form runs the same updates; config 3
    reports the mixed form's error and mask mismatches against the FP64 form
    (the FP64 form is held to the oracle by the parity tests; the oracle takes
    minutes per config-3 update on one core)."""
    import torch
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib

    def run(wl, prec, n_warm, n_timed, stage_mode=None):
        p = dict(wl.params)
        if stage_mode is not None:
            p["stage_mode"] = stage_mode
        d = Domain(p, wl.nx_ice, wl.ny_ice, wl.dx, precision=prec)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        t = 0.0
        for _ in range(n_warm):
            t += wl.dtt
            d.update(wl.H_final, t, b)
        torch.cuda.synchronize()
        a = time.perf_counter()
        for _ in range(n_timed):
            t += wl.dtt
            d.update_async(0, t, b)
        d.synchronize()
        secs = time.perf_counter() - a
        out = {k: d.field(k) for k in ("w", "maskocean", "maskgrounded", "maskcontinent")}
        cells = d.nx * d.ny
        d.close()
        return n_timed * wl.dtt / 1000.0 / secs, secs, out, cells

    def cpu(wl, n_timed, stage_mode=None):
        from oracle import oracle as O
        O.set_threads(1)
        p = dict(wl.params)
        if stage_mode is not None:
            p["stage_mode"] = stage_mode
        m = O.Model(p, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        f = wl.padded_fields(m.nx, m.ny)
        if f:
            m.set_fields(**f)
        bo = O.make_bsl()
        m.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, bo)
        t = wl.dtt
        m.update(wl.H_final, t, bo)
        a = time.perf_counter()
        for _ in range(n_timed):
            t += wl.dtt
            m.update(wl.H_final, t, bo)
        secs = time.perf_counter() - a
        m.close()
        return n_timed * wl.dtt / 1000.0 / secs

    res = {}
    cases = [("config1", W.config1(128), 0, 3, 100, 20), ("config2", W.config2(n=256), None, 3, 30, 2)]
    for name, wl, sm, nw, nt, nc in cases:
        k64, s64, o64, cells = run(wl, 0, nw, nt, sm)
        k32, s32, o32, _ = run(wl, 1, nw, nt, sm)
        err = float(np.abs(o32["w"] - o64["w"]).max() / max(np.abs(o64["w"]).max(), 1e-300))
        res[name] = {"cells": cells, "updates_timed": nt, "fp64_kyr_s": k64, "mixed_kyr_s": k32,
                     "mixed_over_fp64": k32 / k64, "err_mixed_vs_fp64": err,
                     "cpu_oracle_1core_kyr_s": cpu(wl, nc, sm)}
    wl = W.config3()
    k64, s64, o64, cells = run(wl, 0, 2, 4)
    k32, s32, o32, _ = run(wl, 1, 2, 4)
    wmax = max(np.abs(o64["w"]).max(), 1e-300)
    res["config3"] = {"cells": cells, "updates_timed": 4, "fp64_kyr_s": k64, "mixed_kyr_s": k32,
                      "mixed_over_fp64": k32 / k64,
                      "err_mixed_vs_fp64": {"max_rel": float(np.abs(o32["w"] - o64["w"]).max() / wmax),
                                            "rms_rel": float(np.sqrt(np.mean((o32["w"] - o64["w"]) ** 2)) / wmax)},
                      "mask_mismatch": {m: int(np.sum(o32[m] != o64[m]))
                                        for m in ("maskocean", "maskgrounded", "maskcontinent")},
                      "cpu_oracle_1core_kyr_s": None}
    return res


def horizons_leg(oracle_threads=None):
    """Configurations 1-3 to their stated end times in both forms on the
    GPU: configuration 1 (128^2, reference-compatible Tsit5) to 50 kyr with
    the output every 1 kyr, configuration 2 (256^2, RK4 true stages, dt =
    1 yr) to 20 kyr, configuration 3 (512 x 1024, interactive sea level,
    reference-compatible Tsit5) to 10 kyr.  Wall time and simulated kyr/s
    of each form, the mixed form's difference from the FP64 form at the end
    (configuration 1: at every output), mask mismatches, and configuration
    1 at 50 kyr against the oracle (every host core; the frozen RHS of the
    reference's stages evaluated once per attempt, bit-identical)."""
    from fastisostasy_gb300 import workloads as W
    from fastisostasy_gb300.isostasy import Domain
    from fastisostasy_gb300 import _lib

    def run(wl, prec, stage_mode, t_end, out_every):
        p = dict(wl.params)
        if stage_mode is not None:
            p["stage_mode"] = stage_mode
        d = Domain(p, wl.nx_ice, wl.ny_ice, wl.dx, precision=prec)
        f = wl.padded_fields(d.nx, d.ny)
        if f:
            d.set_fields(**f)
        b = _lib.FiBsl()
        b.method, b.constant_ocean_surface = 0, 1
        b.A_ocean_pd = b.A_ocean_now = 3.625e14
        d.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        a = time.perf_counter()
        t = wl.dtt
        d.update(wl.H_final, t, b)
        outs = []
        n = int(round(t_end / wl.dtt))
        for k in range(2, n + 1):
            t = k * wl.dtt
            d.update_async(0, t, b)
            if out_every and (k * wl.dtt) % out_every == 0:
                outs.append(d.field("w"))   # waits for the update
        d.synchronize()
        secs = time.perf_counter() - a
        sc = d.scalars()
        res = {k: d.field(k) for k in ("w", "maskocean", "maskgrounded", "maskcontinent")}
        d.close()
        return secs, res, outs, sc

    out = {}
    cases = [("config1", W.config1(128), 0, 50e3, 1000.0), ("config2", W.config2(n=256), None, 20e3, None),
             ("config3", W.config3(), None, 10e3, None)]
    for name, wl, sm, t_end, every in cases:
        s64, r64, o64, sc64 = run(wl, 0, sm, t_end, every)
        s32, r32, o32, sc32 = run(wl, 1, sm, t_end, every)
        wmax = max(np.abs(r64["w"]).max(), 1e-300)
        e = {"t_end_yr": t_end, "fp64_s": s64, "mixed_s": s32, "fp64_kyr_s": t_end / 1e3 / s64,
             "mixed_kyr_s": t_end / 1e3 / s32,
             "err_mixed_vs_fp64_end": {"max_rel": float(np.abs(r32["w"] - r64["w"]).max() / wmax),
                                       "rms_rel": float(np.sqrt(np.mean((r32["w"] - r64["w"]) ** 2)) / wmax)},
             "mask_mismatch_end": {m: int(np.sum(r32[m] != r64[m]))
                                   for m in ("maskocean", "maskgrounded", "maskcontinent")},
             "steps": {"fp64": [sc64["n_accept"], sc64["n_reject"]], "mixed": [sc32["n_accept"], sc32["n_reject"]]}}
        if o64:
            e["err_mixed_vs_fp64_outputs_max"] = max(float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
                                                     for a, b in zip(o32, o64))
        if name == "config1":
            from oracle import oracle as O
            O.set_threads(oracle_threads or os.cpu_count() or 1)
            O.set_reuse_frozen(True)
            m = O.Model(dict(wl.params, stage_mode=0), wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
            f = wl.padded_fields(m.nx, m.ny)
            if f:
                m.set_fields(**f)
            bo = O.make_bsl()
            m.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, bo)
            a = time.perf_counter()
            for k in range(1, int(round(t_end / wl.dtt)) + 1):
                rc = m.update(wl.H_final, k * wl.dtt, bo)
                if rc:
                    break
            so = m.scalars()
            wo = m.field("w")
            e["oracle"] = {"s": time.perf_counter() - a, "rc": int(rc), "steps": [so["n_accept"], so["n_reject"]],
                           "fp64_vs_oracle_max_rel": float(np.abs(r64["w"] - wo).max() / max(np.abs(wo).max(), 1e-300)),
                           "mixed_vs_oracle_max_rel": float(np.abs(r32["w"] - wo).max() / max(np.abs(wo).max(), 1e-300))}
            m.close()
            O.set_reuse_frozen(False)
        out[name] = e
    return {"horizons": out}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    O.set_threads(threads)
    O.set_smooth_convolution(True)
    wl = workload(stage_mode=1)
    m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
    m.set_fields(**wl.padded_fields(m.nx, m.ny))
    bo = O.make_bsl()
    m.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bo)
    t = 0.0
    for _ in range(args.warmup):
        t += wl.dtt
        m.update(wl.H_final, t, bo)
    a = time.perf_counter()
    for _ in range(args.steps):
        t += wl.dtt
        m.update(wl.H_final, t, bo)
    secs = time.perf_counter() - a
    val = args.steps * wl.dtt / 1000.0 / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "kyr/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "FP64", "stage_mode": "true stages", "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": val, "unit": "kyr/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
                         "sample": "%d coupling steps (%d x 40 RHS + 2 convolutions at 1024^2, the smallest "
                                   "smooth size >= 2n-1), OpenMP %d threads" % (args.steps, args.steps, threads)},
        "e2e": {"value": val, "unit": "kyr/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-samples", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--no-oracle", action="store_true", help="skip the err_vs_oracle leg")
    ap.add_argument("--ensemble-members", type=int, default=256)
    ap.add_argument("--ensemble-updates", type=int, default=10)
    ap.add_argument("--groups", type=int, default=2, help="stiffness groups of --only ensemble-true")
    ap.add_argument("--ensemble-mode", default="graph", choices=["graph", "streams"],
                    help="batched graphs or per-member streams for --only ensemble-true")
    ap.add_argument("--scale-sizes", default="1024,2048", help="grid sizes of --only scale")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--only", choices=["ensemble", "ensemble-true", "ensemble-full", "serve", "configs", "horizons",
                                       "scale", "oracle",
                                       "engine-trace"],
                    help="run one secondary leg alone and print its JSON (for profiling), not a bench line")
    ap.add_argument("--lean", action="store_true",
                    help="mixed form only, no profile / e2e / CPU legs (for ncu captures); prints the timing only")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    from fastisostasy_gb300 import _lib
    _lib.load()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    results = {}
    if args.only == "ensemble":
        print(json.dumps({"ensemble": ensemble_leg(args.ensemble_members, args.ensemble_updates)}))
        return 0
    if args.only == "serve":
        print(json.dumps({"serve": serve_leg(n_req=args.serve_requests)}))
        return 0
    if args.only == "ensemble-full":
        print(json.dumps({"ensemble_full": ensemble_full_leg()}))
        return 0
    if args.only == "ensemble-true":
        print(json.dumps({"ensemble_true": ensemble_true_leg(groups=args.groups, mode=args.ensemble_mode)}))
        return 0
    if args.only == "engine-trace":
        print(json.dumps({"engine_trace": engine_trace_leg()}))
        return 0
    if args.only == "oracle":
        print(json.dumps({"err_vs_oracle": oracle_leg()}))
        return 0
    if args.only == "configs":
        print(json.dumps({"configs": configs_leg()}))
        return 0
    if args.only == "horizons":
        print(json.dumps(horizons_leg()))
        return 0
    if args.only == "scale":
        print(json.dumps({"scale": scale_leg(tuple(int(v) for v in args.scale_sizes.split(",")))}))
        return 0
    if args.lean:
        dom, wl, b = make_domain(1)
        ms, _, _, _, _ = run_resident(dom, wl, b, args.steps, args.warmup, flush)
        print(json.dumps({"lean": True, "ms_per_step": sum(ms) / len(ms), "steps": args.steps}))
        dom.close()
        return 0
    for prec in (0, 1):
        dom, wl, b = make_domain(prec)
        barrier()
        ms, launches, clocks, _, t_end = run_resident(dom, wl, b, args.steps, args.warmup, flush,
                                                      sampler_index=local if prec == 1 else None)
        barrier()
        tot = sum(ms)
        from fastisostasy_gb300 import replicas
        tot = replicas.max_over_ranks(tot, device="cuda")   # slowest replica
        results[prec] = {"dom": dom, "wl": wl, "b": b, "ms": tot / args.steps, "launches": launches,
                         "clocks": clocks, "w": dom.field("w"), "t": t_end}
    kyr = lambda ms_step: ws * (DTT / 1000.0) / (ms_step / 1000.0)
    r64, r32 = results[0], results[1]
    w64, w32 = r64["w"], r32["w"]
    err_max = float(np.abs(w32 - w64).max() / np.abs(w64).max())
    err_rms = float(np.sqrt(np.mean((w32 - w64) ** 2)) / np.abs(w64).max())

    # per-kernel CUDA-event timing pass (same workload, same step count) for the roofline
    dom, wl, b = r32["dom"], r32["wl"], r32["b"]
    _, _, _, prof, t_now = run_resident(dom, wl, b, args.steps, 0, flush, t0=r32["t"], profile=True)
    peak, peak_kind = peaks()
    dominant = max(prof.items(), key=lambda kv: kv[1][0])[0]
    tot_ms, cnt = prof[dominant]
    alg = algorithmic_bytes(dominant, dom, 1, 1)
    achieved = alg / (tot_ms / cnt / 1000.0) / 1e9 if alg else None
    upd = update_bytes(dom, 1)
    shares = {k: round(v[0] / sum(x[0] for x in prof.values()), 4) for k, v in prof.items()}

    # end to end through fi_update with host arrays (mixed form)
    e2e_secs, h2d, d2h = run_e2e(dom, wl, b, args.steps, 1, flush, t_now)
    t_now += wl.dtt * (args.steps + 1)
    # device-resident updates with an asynchronous isos%out snapshot after
    # every update (fi_output_async) against the same updates without
    outp = output_leg(dom, wl, b, args.steps, t_now)

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, secs = cpu_baseline(args.cpu_samples, threads=1, stage_mode=1)
        cpu = {"value": v, "unit": "kyr/s", "cores": 1, "kind": "port", "cpu": cpu_model(),
               "sample": "%d coupling steps of the same workload (%d x 40 RHS + 2 convolutions at 1024^2, the "
                         "smallest smooth size >= 2n-1), %.1f s, 1 thread (the reference is serial)"
                         % (args.cpu_samples, args.cpu_samples, secs)}

    ens = serve = cfgs = orc = None
    if rank == 0 and not args.no_oracle:
        orc = oracle_leg()
    if not args.no_configs:
        cfgs = configs_leg()
    if not args.no_ensemble:
        ens = ensemble_leg(args.ensemble_members, args.ensemble_updates)
    if not args.no_serve:
        serve = serve_leg(n_req=args.serve_requests)

    if rank == 0:
        line = {
            "metric": METRIC, "value": kyr(r32["ms"]), "unit": "kyr/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r32["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "mixed FP32/FP64", "stage_mode": "true stages",
                       "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas" if ws > 1 else "1 GPU"},
            "fp64": {"value": kyr(r64["ms"]), "unit": "kyr/s", "ms_per_step": r64["ms"], "dtype": "f64"},
            "mixed_over_fp64": r64["ms"] / r32["ms"],
            "err_vs_fp64": {"max_rel": err_max, "rms_rel": err_rms,
                            "after_steps": args.warmup + args.steps},
            "err_vs_oracle": orc,
            "cell_steps_per_s": ws * N_CELLS * N_CELLS * (DTT / DT) / (r32["ms"] / 1000.0),
            "e2e": {"value": kyr(1000.0 * e2e_secs / args.steps), "unit": "kyr/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": ncu_traffic(dominant),
                         "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg,
                         "avg_launch_us": 1000.0 * tot_ms / cnt, "kernel_time_shares": shares,
                         "whole_update": {"algorithmic_bytes": upd,
                                          "achieved": upd / (r32["ms"] / 1000.0) / 1e9,
                                          "frac": upd / (r32["ms"] / 1000.0) / 1e9 / peak},
                         "l2": l2_line(dominant, 1000.0 * tot_ms / cnt)},
            "output_async": outp,
            "cpu_baseline": cpu,
            "configs": cfgs,
            "ensemble": ens,
            "serve": serve,
            "clocks": r32["clocks"],
            "gpu_launches": r32["launches"],
        }
        print(json.dumps(line))
    for r in results.values():
        r["dom"].close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
