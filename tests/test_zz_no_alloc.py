"""fi_lvelva_static: calc_lvelva for callers that may not allocate device
memory once running, checked against fi_lvelva and the oracle.

Some callers cannot allocate: a coupled model that divides the GPU's memory
among its components at start-up, or a time loop that cannot afford the
device-wide synchronisation of cudaFree.  The entry point computes in one
static device scratch array instead.  This file's name sorts last so that it
also runs after every other GPU test has used the device.  Its device arrays
are made by torch: the test may allocate, the entry point under test must
not, which the free-memory check below verifies.
"""
import json
import os

import numpy as np
import pytest

from fastisostasy_gb300 import _lib
from fastisostasy_gb300.isostasy import Domain
from harness import rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-10


def _case(nx, ny, seed, even_R):
    rng = np.random.default_rng(seed)
    D = 1e24 * (1 + rng.random((ny, nx)))
    eta = 1e21 * (1 + rng.random((ny, nx)))
    R = np.ones((ny, nx)) if even_R else 1 + 0.2 * rng.random((ny, nx))
    mask = (rng.random((ny, nx)) > 0.15).astype(np.uint8)
    return D, eta, R, mask


def _inputs(nx, ny, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((ny, nx)) * 100, rng.standard_normal((ny, nx)) * 1e5


def _params(nx, ny):
    with open(os.path.join(GOLDEN, "params_test1d.json")) as fh:
        p = json.load(fh)
    p.update(nx_target=nx if nx != ny else 0, ny_target=ny if nx != ny else 0)
    return p


class Static:
    """Device copies of one grid's fields and a caller of fi_lvelva_static."""

    def __init__(self, torch, mask, D, eta, kappa, R, dxm=None, dym=None):
        self.torch = torch
        self.dev = torch.device("cuda", 0)
        t = self.to
        self.mask, self.D, self.eta, self.kap, self.R = t(mask.astype(np.uint8)), t(D), t(eta), t(kappa), t(R)
        self.dxm = t(dxm) if dxm is not None else None
        self.dym = t(dym) if dym is not None else None
        self.ny, self.nx = D.shape
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream

    def to(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)

    def call(self, d_w, d_cf, d_out, dx, dy, g, nu, spy):
        ptr = lambda a: a.data_ptr() if a is not None else None
        return _lib.load().fi_lvelva_static(ptr(d_w), ptr(d_cf), ptr(self.mask), ptr(self.D), ptr(self.eta),
                                            ptr(self.kap), ptr(self.R), ptr(self.dxm), ptr(self.dym), self.nx,
                                            self.ny, dx, dy, g, nu, spy, ptr(d_out), self.stream)

    def run(self, w, cf, dx, dy, g, nu, spy):
        d_w, d_cf = self.to(w), self.to(cf)
        d_out = self.torch.full((self.ny, self.nx), float("nan"), dtype=self.torch.float64, device=self.dev)
        assert self.call(d_w, d_cf, d_out, dx, dy, g, nu, spy) == _lib.FI_OK
        self.torch.cuda.synchronize(self.dev)
        return d_out.cpu().numpy()


@pytest.mark.parametrize("nx,ny,even,distorted", [(48, 80, False, False), (256, 256, True, False),
                                                  (96, 96, False, True)])
def test_lvelva_static_matches_lvelva(nx, ny, even, distorted):
    """Two calls in a row through the same scratch against fi_lvelva on a
    handle with the same fields; `distorted` passes a projection factor K
    (spacing dx*K, dy*K per cell) to both."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    p = _params(nx, ny)
    dx = 50e3
    K = None
    if distorted:
        yy = np.linspace(-1.0, 1.0, ny)[:, None] * np.ones((1, nx))
        K = 1.0 + 0.08 * yy ** 2 + 0.02 * np.sin(np.linspace(0, 3, nx))[None, :]
    dom = Domain(p, nx, ny, dx, K=K, precision=0)
    assert (dom.nx, dom.ny) == (nx, ny)
    D, eta, R, mask = _case(nx, ny, 11 * nx + ny, even)
    dom.set_fields(D_lith=D, eta_eff=eta, R=R, maskactive=mask)
    spy = dom.scalars()["sec_per_year"]
    st = Static(torch, dom.field("maskactive"), dom.field("D_lith"), dom.field("eta_eff"), dom.field("kappa"),
                dom.field("R"), dxm=None if K is None else dx * K, dym=None if K is None else dx * K)
    for call in range(2):
        w, cf = _inputs(nx, ny, 1000 * call + nx)
        want = dom.lvelva(w, cf)
        got = st.run(w, cf, dx, dx, p["g"], p["nu"], spy)
        assert np.isfinite(got).all()
        assert rel(got, want) <= TOL64, (call, rel(got, want))
    if distorted:
        # the spacing matters: the uniform-spacing result is far from it
        st.dxm = st.dym = None
        assert rel(st.run(w, cf, dx, dx, p["g"], p["nu"], spy), want) > 1e-4
    dom.close()


@pytest.mark.parametrize("nx,ny", [(254, 44), (44, 242)])
def test_lvelva_static_prime_lengths_match_oracle(nx, ny):
    """Lengths with large prime factors (a 127-point row transform; 242 =
    2 * 11^2), which a handle never builds unpadded, against the oracle."""
    torch = pytest.importorskip("torch")
    p = _params(nx, ny)
    dx = 40e3
    D, eta, R, mask = _case(nx, ny, nx + 3 * ny, False)
    kap = O.kappa(nx, ny, dx, dx)
    spy = float(np.float32(3600.0) * np.float32(24.0) * np.float32(365.25))
    st = Static(torch, mask, D, eta, kap, R)
    dxm = np.full((ny, nx), dx)
    for call in range(2):
        w, cf = _inputs(nx, ny, 7 + call)
        want = O.lvelva(w, cf, mask, p["g"], p["nu"], D, eta, R, kap, dxm, dxm, spy)
        got = st.run(w, cf, dx, dx, p["g"], p["nu"], spy)
        assert rel(got, want) <= TOL64, (call, rel(got, want))


def test_lvelva_static_allocates_nothing():
    """After a first call (which loads the library's device code), further
    calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    nx = ny = 128
    p = _params(nx, ny)
    dx = 50e3
    D, eta, R, mask = _case(nx, ny, 5, True)
    st = Static(torch, mask, D, eta, O.kappa(nx, ny, dx, dx), R)
    w, cf = _inputs(nx, ny, 3)
    d_w, d_cf = st.to(w), st.to(cf)
    d_out = torch.empty((ny, nx), dtype=torch.float64, device=st.dev)
    assert st.call(d_w, d_cf, d_out, dx, dx, p["g"], p["nu"], 3.15576e7) == _lib.FI_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(8):
        assert st.call(d_w, d_cf, d_out, dx, dx, p["g"], p["nu"], 3.15576e7) == _lib.FI_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0


def test_lvelva_static_refuses_oversize():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n = _lib.FI_STATIC_MAX_N + 2
    buf = torch.zeros(n * n, dtype=torch.float64, device="cuda:0")
    m = torch.zeros(n * n, dtype=torch.uint8, device="cuda:0")
    ptr = buf.data_ptr()
    for nx, ny in ((n, 64), (64, n), (63, 64)):
        rc = L.fi_lvelva_static(ptr, ptr, m.data_ptr(), ptr, ptr, ptr, ptr, None, None, nx, ny, 50e3, 50e3, 9.81,
                                0.28, 3.15576e7, ptr, None)
        assert rc == _lib.FI_E_SIZE
    # spacing fields: both or neither
    rc = L.fi_lvelva_static(ptr, ptr, m.data_ptr(), ptr, ptr, ptr, ptr, ptr, None, 64, 64, 50e3, 50e3, 9.81,
                            0.28, 3.15576e7, ptr, None)
    assert rc == _lib.FI_E_ARG
    torch.cuda.synchronize()
