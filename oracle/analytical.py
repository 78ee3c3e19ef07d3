"""Analytical ELVA disk (Bueler et al. 2007, eq. 17) — test infrastructure.

Restates ``isosbench_elva_disk`` (src/isostasy_benchmarks.f90:74-127) and
``calc_analytical_viscous_disk[_params]`` (:131-280):

    u(r, t) = int_0^0.1 rho_i g h0 r0 (exp(-beta t / (2 eta k)) - 1)
                         J1(k r0) J0(k r) / beta  dk,   beta = rho_m g + D k^4

integrated over [0, 0.1] (the reference uses adaptive 6-point Gauss-Legendre
with tol 1e-6 on sub-intervals of width 1e-3; here a composite Gauss-Legendre
rule with panels of 2e-7 on [0, 1e-3], where J1(k r0) oscillates, and 1e-4
beyond), remapped radially onto the grid and shifted by the mean of the four
corners.  The time unit is 365*24*3600 s per year
(:338).
"""
import numpy as np
from scipy.special import j0, j1


def radial_profile(radii, r0, h0, eta, D, rho_ice, rho_m, g, time_yr, npts=8):
    t_sec = time_yr * 365 * 24 * 3600
    xg, wg = np.polynomial.legendre.leggauss(npts)
    ks = np.concatenate([np.linspace(0.0, 1e-3, 5001), np.linspace(1e-3, 0.1, 991)[1:]])
    out = np.zeros(len(radii))
    for a, b in zip(ks[:-1], ks[1:]):
        k = 0.5 * (b - a) * xg + 0.5 * (a + b)
        w = 0.5 * (b - a) * wg
        beta = rho_m * g + D * k ** 4
        base = rho_ice * g * h0 * r0 * (np.exp(-beta * t_sec / (2 * eta * k)) - 1.0) * j1(k * r0) / beta
        out += (w[None, :] * base[None, :] * j0(np.outer(radii, k))).sum(axis=1)
    return out


def elva_disk(nx, ny, dx, r0, h0, eta, D, rho_ice, rho_m, g, time_yr):
    """Field (ny, nx) as isosbench_elva_disk writes it."""
    ic, jc = (nx - 1) // 2 + 1, (ny - 1) // 2 + 1
    i = np.arange(1, nx + 1)
    j = np.arange(1, ny + 1)
    dist = np.sqrt((dx * (i[None, :] - ic)) ** 2 + (dx * (j[:, None] - jc)) ** 2)
    nl = int(max(nx, ny) * np.sqrt(2.0) / 2) + 2
    rad = dx * np.arange(nl)
    lr = np.floor(dist / dx).astype(int)          # r(l) <= dist < r(l+1)
    prof = radial_profile(rad, r0, h0, eta, D, rho_ice, rho_m, g, time_yr)
    w = prof[lr]
    return w - 0.25 * (w[0, 0] + w[-1, -1] + w[-1, 0] + w[0, -1])
