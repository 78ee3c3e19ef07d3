"""Independent numpy restatement of pieces of the LV-ELVA path.

Used by the CPU tests to pin the C oracle: transforms are built from their
definitions (explicit cas / exp matrices, numpy's pocketfft), derivatives
from array slicing.  Citations are to the reference project's files.
Arrays are (ny, nx) C-order == Fortran (nx, ny) column-major.
"""
import numpy as np

PI_LIT = float(np.float32(3.14159265359))   # src/isostasy_defs.f90:8


def cas_matrix(n):
    k = np.arange(n)
    a = 2 * np.pi * np.outer(k, k) / n
    return np.cos(a) + np.sin(a)


def dht2d(a):
    """FFTW_DHT x FFTW_DHT (unnormalised): H = Cy @ a @ Cx (a is (ny, nx))."""
    ny, nx = a.shape
    return cas_matrix(ny) @ a @ cas_matrix(nx).T


def d_x(u, dx):     # src/finite_differences.f90:17-41
    d = np.zeros_like(u)
    d[:, 1:-1] = (u[:, 2:] - u[:, :-2]) / (2 * dx[:, 1:-1])
    d[:, -1] = (u[:, -1] - u[:, -2]) / dx[:, -1]
    d[:, 0] = (u[:, 1] - u[:, 0]) / dx[:, 0]
    return d


def d_y(u, dy):     # :43-67
    return d_x(u.T, dy.T).T


def d_xx(u, dx):    # :70-94, note the dx(1,:) quirk on the last row
    d = np.zeros_like(u)
    d[:, 1:-1] = (u[:, 2:] - 2 * u[:, 1:-1] + u[:, :-2]) / (dx[:, 1:-1] * dx[:, 1:-1])
    d[:, 0] = (u[:, 2] - 2 * u[:, 1] + u[:, 0]) / (dx[:, 0] * dx[:, 0])
    d[:, -1] = (u[:, -1] - 2 * u[:, -2] + u[:, -3]) / (dx[:, 0] * dx[:, 0])
    return d


def d_yy(u, dy):    # :96-120 (no quirk in y)
    d = np.zeros_like(u)
    d[1:-1, :] = (u[2:, :] - 2 * u[1:-1, :] + u[:-2, :]) / (dy[1:-1, :] * dy[1:-1, :])
    d[0, :] = (u[2, :] - 2 * u[1, :] + u[0, :]) / (dy[0, :] * dy[0, :])
    d[-1, :] = (u[-1, :] - 2 * u[-2, :] + u[-3, :]) / (dy[-1, :] * dy[-1, :])
    return d


def kappa(nx, ny, dx, dy):   # src/lv_elva.f90:442-481
    mu_x = 2.0 * PI_LIT / ((nx - 1) * dx)
    mu_y = 2.0 * PI_LIT / ((ny - 1) * dy)
    i = np.arange(1, nx + 1)
    j = np.arange(1, ny + 1)
    ic, jc = (nx - 1) // 2 + 1, (ny - 1) // 2 + 1
    p = np.where(i <= ic, mu_x * (i - 1), mu_x * (nx - i + 1))
    q = np.where(j <= jc, mu_y * (j - 1), mu_y * (ny - j + 1))
    k = np.sqrt(p[None, :] ** 2 + q[:, None] ** 2)
    k[0, 0] = (k[1, 0] + k[0, 1]) / 2.0
    return k


def corners(x):
    return 0.25 * (x[0, 0] + x[-1, -1] + x[-1, 0] + x[0, -1])


def lvelva(w, canom_full, mask, g, nu, D, eta, R, kap, dxm, dym, spy):
    """calc_lvelva, src/lv_elva.f90:31-126."""
    w_x = d_x(w, dxm)
    w_xy = d_y(w_x, dym)
    w_xx = d_xx(w, dxm)
    w_yy = d_yy(w, dym)
    Mxx = -D * (w_xx + nu * w_yy)
    Myy = -D * (w_yy + nu * w_xx)
    Mxy = -D * (1.0 - nu) * w_xy
    Mxy_xy = d_y(d_x(Mxy, dxm), dym)
    Mx_xx = d_xx(Mxx, dxm)
    My_yy = d_yy(Myy, dym)
    p = np.where(mask, -g * canom_full, 0.0)
    f = (p + Mx_xx + 2.0 * Mxy_xy + My_yy) / (2.0 * eta)
    fh = dht2d(f) / (kap * R)
    out = dht2d(fh) / (w.size * 1.0)
    out = out - corners(out)
    return out * spy


def linear_conv_crop(kernel, inp):
    """precomputed_fftconvolution, src/convolutions.f90:59-91, as a direct
    linear convolution (the (2n-1)^2 circular one has no wrap-around)."""
    ny, nx = inp.shape
    M = 2 * max(nx, ny) - 1
    full = np.real(np.fft.ifft2(np.fft.fft2(kernel, (M, M)) * np.fft.fft2(inp, (M, M))))
    full = full - 0.25 * (full[0, 0] + full[M - 1, M - 1] + full[M - 1, 0] + full[0, M - 1])
    j1, i1 = ny // 2, nx // 2
    return full[j1 - 1:j1 - 1 + ny, i1 - 1:i1 - 1 + nx]
