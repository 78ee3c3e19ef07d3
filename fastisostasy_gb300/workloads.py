"""Synthetic LV-ELVA workloads (seeded), the inputs of the parity cases and
benchmarks.

Each builder returns a ``Workload``: parameters, ice grid size and spacing,
the padded-grid fields a caller would pass through ``fi_set_fields``, the
initial bed and ice, and an ice-thickness history ``H_at(t)``.  The
reference's own test set-ups (tests/test_isostasy.f90:66-345 and
par/test_isostasy_test*.nml) define the disc experiments; the rest are the
synthetic stand-ins for data the reference reads from files that are not
part of its repository (isostasy_data).
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Optional

import numpy as np

from . import params as P


@dataclasses.dataclass
class Workload:
    name: str
    params: dict
    nx_ice: int
    ny_ice: int
    dx: float
    z_bed: np.ndarray                      # (ny_ice, nx_ice)
    H_final: np.ndarray                    # (ny_ice, nx_ice)
    dtt: float = 10.0                      # coupling interval [yr]
    t_end: float = 1000.0
    switch_on: float = 1e-9                # load history: 0 before, H_final after
    fields: dict = dataclasses.field(default_factory=dict)   # padded-grid overrides
    fields_fn: Optional[Callable] = None   # (nx, ny, dx) -> dict of padded fields
    bsl: dict = dataclasses.field(default_factory=lambda: dict(method=0, bsl_init=0.0, A_ocean_pd=3.625e14))

    def H_at(self, t: float) -> np.ndarray:
        """interp_2d over the two-slice history of the disc tests
        (tests/test_isostasy.f90:233-239, src/isos_utils.f90:460-495)."""
        if t < self.switch_on:
            if t <= 0.0:
                return np.zeros_like(self.H_final)
            return self.H_final * (t / self.switch_on)
        return self.H_final

    def padded_fields(self, nx: int, ny: int) -> dict:
        f = dict(self.fields)
        if self.fields_fn is not None:
            f.update(self.fields_fn(nx, ny, self.dx))
        return f


def disc(nx, ny, dx, r0=1000e3, h0=1000.0):
    """Centred ice disc on the ice grid (tests/test_isostasy.f90:222-231)."""
    xc = (np.arange(nx) - (nx - 1) / 2.0) * dx
    yc = (np.arange(ny) - (ny - 1) / 2.0) * dx
    return np.where(xc[None, :] ** 2 + yc[:, None] ** 2 <= r0 ** 2, h0, 0.0)


def ref_test(nml_path: str, nx=121, dx=50e3, t_end=50e3, **over) -> Workload:
    """A reference disc experiment (test1*/test3*) from its namelist file."""
    p = P.load(nml_path)
    p.update(over)
    H = disc(nx, nx, dx)
    return Workload(name="ref_" + nml_path.rsplit("/", 1)[-1], params=p, nx_ice=nx, ny_ice=nx,
                    dx=dx, z_bed=np.full((nx, nx), 1e6), H_final=H, t_end=t_end)


def config1(n=128, t_end=50e3) -> Workload:
    """Uniform ELVA disc, 4000 km at 31.25 km (128^2), Tsit5, D = 1e25."""
    dx = 4000e3 / n * (128 / 128)
    dx = 31.25e3 if n == 128 else 4000e3 / n
    p = dict(P.DEFAULTS)
    p.update(nu=0.25, rho_uppermantle=3300.0, rho_ice=910.0, dt_method=2, E=66.0)
    # D = 1e25 set directly through the rigidity field
    H = disc(n, n, dx)
    def fields_fn(nx, ny, d):
        return {"D_lith": np.full((ny, nx), 1e25)}
    return Workload(name="config1_%d" % n, params=p, nx_ice=n, ny_ice=n, dx=dx,
                    z_bed=np.zeros((n, n)), H_final=H, t_end=t_end, fields_fn=fields_fn)


def gaussian_lithosphere_D(nx, ny, dx, He0=150e3, amp=100e3, sigma=500e3, E=66.0, nu=0.28):
    """He = He0 - amp exp(-r^2 / (2 sigma^2)) on the padded grid, mapped to D
    with calc_heterogeneous_rigidity's formula (src/isos_utils.f90:90-100)."""
    xc = (np.arange(1, nx + 1) - nx // 2 - 1) * dx    # init_dims, src/isos_utils.f90:221-240
    yc = (np.arange(1, ny + 1) - ny // 2 - 1) * dx
    r2 = xc[None, :] ** 2 + yc[:, None] ** 2
    He = He0 - amp * np.exp(-r2 / (2 * sigma ** 2))
    return E * 1e9 * He ** 3 / (12.0 * (1.0 - nu ** 2))


def config2(n=256, L=3000e3, dt=1.0, dtt=10.0, t_end=20e3, stage_mode=1, elastic=True) -> Workload:
    """Laterally variable LV-ELVA: Gaussian-thinned lithosphere (150 km minus a
    100 km, sigma = 500 km Gaussian), uniform eta = 1e21, disc load, elastic
    and geoid convolutions on, RK4 at fixed dt.

    dt defaults to 1 yr: at dx = 11.7 km and D up to 2e25 N m the flexural
    eigenvalue of the discrete operator is about -1.8 /yr, so RK4 at
    dt = 10 yr (lambda*dt ~ -18) diverges."""
    dx = L / n
    p = dict(P.DEFAULTS)
    p.update(E=66.0, nu=0.28, dt_method=1, dt_init=dt, dt_max=dt, stage_mode=stage_mode,
             include_elastic=int(elastic), heterogeneous_ssh=int(elastic), rho_litho=3200.0,
             rho_uppermantle=3300.0, zl=[150e3], lithosphere=3)
    H = disc(n, n, dx)
    def fields_fn(nx, ny, d):
        return {"D_lith": gaussian_lithosphere_D(nx, ny, d)}
    return Workload(name="config2_%d" % n, params=p, nx_ice=n, ny_ice=n, dx=dx,
                    z_bed=np.full((n, n), 1e6), H_final=H, dtt=dtt, t_end=t_end, fields_fn=fields_fn)


def fractal_field(ny, nx, dx, slope=-2.0, std=600.0, mean=200.0, seed=0):
    """Seeded isotropic fractal field with power spectrum ~ k^slope."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, d=dx)
    ky = np.fft.fftfreq(ny, d=dx)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    k[0, 0] = np.inf
    amp = k ** (slope / 2.0)
    amp[0, 0] = 0.0
    noise = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    f = np.real(np.fft.ifft2(noise * amp))
    f = (f - f.mean()) / f.std()
    return mean + std * f


def config3(nx_ice=336, ny_ice=560, dx=5e3, nx_pad=512, ny_pad=1024, t_end=10e3, seed=3,
            dt_method=2) -> Workload:
    """Greenland-like synthetic domain: fractal bed with an ocean margin,
    parabolic dome masked to land, two-layer mantle (1e20 over 1e21 Pa s,
    boundary 400 km) with frequency-domain lumping, elastic + geoid on,
    interactive sea level, rectangular padding."""
    bed = fractal_field(ny_ice, nx_ice, dx, seed=seed)
    # ocean margin: ramp the bed below sea level over the outer 15 %
    yy, xx = np.meshgrid(np.linspace(-1, 1, ny_ice), np.linspace(-1, 1, nx_ice), indexing="ij")
    edge = np.maximum(np.abs(xx), np.abs(yy))
    bed = bed - 1500.0 * np.clip((edge - 0.7) / 0.3, 0.0, 1.0)
    r = np.sqrt((xx / 0.65) ** 2 + (yy / 0.75) ** 2)
    H = np.where(r < 1.0, 3000.0 * np.sqrt(np.clip(1.0 - r ** 2, 0.0, 1.0)), 0.0)
    H = np.where(bed > -50.0, H, 0.0)
    p = dict(P.DEFAULTS)
    p.update(interactive_sealevel=1, include_elastic=1, heterogeneous_ssh=1, rho_litho=3200.0,
             nl=2, zl=[100e3, 400e3], viscosities=[1e20, 1e21], lumping=5, dt_method=dt_method,
             nx_target=nx_pad, ny_target=ny_pad, min_pad=400e3)
    return Workload(name="config3", params=p, nx_ice=nx_ice, ny_ice=ny_ice, dx=dx, z_bed=bed,
                    H_final=H, t_end=t_end)


def gaussian_random_field(ny, nx, dx, mean=21.0, std=0.5, corr=500e3, seed=0):
    """Squared-exponential-correlated Gaussian random field by FFT filtering."""
    rng = np.random.default_rng(seed)
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=dx)
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    filt = np.exp(-k2 * corr ** 2 / 4.0)
    f = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal((ny, nx))) * filt))
    f = (f - f.mean()) / (f.std() + 1e-300)
    return mean + std * f


def ensemble_member(i: int, stage_mode=1, t_end=10e3) -> Workload:
    """Member i of the 256-member ensemble: n in {128,192,256,384,512}, dx in
    [10, 30] km, log10 eta a Gaussian random field (mean 21, std 0.5,
    correlation 500 km), lithosphere 50-150 km, disc radius 300-1200 km and
    thickness 500-3000 m.  Seeded by the member id."""
    rng = np.random.default_rng(1000 + i)
    n = int(rng.choice([128, 192, 256, 384, 512]))
    dx = float(rng.uniform(10e3, 30e3))
    He = float(rng.uniform(50e3, 150e3))
    r0 = float(rng.uniform(300e3, 1200e3))
    h0 = float(rng.uniform(500.0, 3000.0))
    p = dict(P.DEFAULTS)
    p.update(E=66.0, nu=0.28, zl=[He], dt_method=2, stage_mode=stage_mode, mantle=3)
    H = disc(n, n, dx, r0=r0, h0=h0)
    def fields_fn(nx, ny, d, _i=i):
        return {"eta_eff": 10.0 ** gaussian_random_field(ny, nx, d, seed=_i)}
    return Workload(name="member_%d" % i, params=p, nx_ice=n, ny_ice=n, dx=dx,
                    z_bed=np.full((n, n), 1e6), H_final=H, t_end=t_end, fields_fn=fields_fn)


SERVE_SIZES = (64, 128, 256, 512, 1024)
SERVE_WEIGHTS = (0.3, 0.3, 0.2, 0.15, 0.05)


def serve_sizes(n_req: int, seed: int = 77) -> list:
    """Grid sizes of a stream of n_req requests in SERVE_WEIGHTS proportions
    by quota (largest remainders), in a seeded random order: every size
    appears at its weight even in a short stream (a draw of 48 can miss the
    5 % of 1024^2 requests entirely)."""
    quota = [w * n_req for w in SERVE_WEIGHTS]
    counts = [int(q) for q in quota]
    for k in sorted(range(len(quota)), key=lambda k: counts[k] - quota[k])[: n_req - sum(counts)]:
        counts[k] += 1
    sizes = [n for n, c in zip(SERVE_SIZES, counts) for _ in range(c)]
    np.random.default_rng(seed).shuffle(sizes)
    return [int(v) for v in sizes]


def serve_request(i: int, horizon_scale: float = 0.01, dx: float = 25e3, n: Optional[int] = None) -> Workload:
    """Request i of the serving stream: n drawn from SERVE_SIZES with
    SERVE_WEIGHTS, seeded random-field mantle viscosity (log10 eta: mean 21,
    std 0.25, correlation 500 km) and lithosphere thickness (mean 85 km, std
    15 km, clipped to 50-120 km, mapped to rigidity with E = 66 GPa,
    nu = 0.28), a disc or a parabolic dome load, horizon log-uniform in
    1-100 kyr times `horizon_scale` (`n` overrides the drawn size, for
    quota-sized streams).  RK4 with true stages at dt = 1 yr,
    coupling every 10 yr; the spacing keeps dt = 1 yr inside RK4's stability
    region for every draw."""
    rng = np.random.default_rng(5000 + i)
    drawn = int(rng.choice(SERVE_SIZES, p=SERVE_WEIGHTS))
    n = drawn if n is None else int(n)
    horizon = float(np.exp(rng.uniform(np.log(1e3), np.log(1e5)))) * horizon_scale
    horizon = max(10.0, 10.0 * np.ceil(horizon / 10.0))
    L = n * dx
    r0 = float(rng.uniform(0.15, 0.35)) * L
    h0 = float(rng.uniform(500.0, 3000.0))
    dome = bool(rng.random() < 0.5)
    xc = (np.arange(n) - (n - 1) / 2.0) * dx
    r = np.sqrt(xc[None, :] ** 2 + xc[:, None] ** 2)
    H = np.where(r <= r0, h0 * (np.sqrt(np.clip(1.0 - (r / r0) ** 2, 0.0, 1.0)) if dome else 1.0), 0.0)
    p = dict(P.DEFAULTS)
    p.update(E=66.0, nu=0.28, dt_method=1, dt_init=1.0, dt_max=1.0, stage_mode=1, lithosphere=3, mantle=3)
    seed = 7000 + i

    def fields_fn(nx, ny, d, _s=seed):
        He = np.clip(gaussian_random_field(ny, nx, d, mean=85e3, std=15e3, seed=_s), 50e3, 120e3)
        D = 66.0 * 1e9 * He ** 3 / (12.0 * (1.0 - 0.28 ** 2))
        eta = 10.0 ** gaussian_random_field(ny, nx, d, mean=21.0, std=0.25, seed=_s + 1)
        return {"D_lith": D, "eta_eff": eta}
    return Workload(name="request_%d" % i, params=p, nx_ice=n, ny_ice=n, dx=dx, z_bed=np.full((n, n), 1e6),
                    H_final=H, dtt=10.0, t_end=horizon, fields_fn=fields_fn)
