"""fi_lvelva_static (static device scratch, no allocation) against fi_lvelva.

The file name sorts last so that the entry point also runs after every other
GPU test has used the device.  Device arrays are made by torch here: the test
may allocate, the entry point under test does not.
"""
import json
import os

import numpy as np
import pytest

from fastisostasy_gb300 import _lib
from fastisostasy_gb300.isostasy import Domain
from harness import rel

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


@pytest.mark.parametrize("nx,ny,even", [(48, 80, False), (256, 256, True)])
def test_lvelva_static_matches_lvelva(nx, ny, even):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    L = _lib.load()
    with open(os.path.join(GOLDEN, "params_test1d.json")) as fh:
        p = json.load(fh)
    p.update(nx_target=nx if nx != ny else 0, ny_target=ny if nx != ny else 0)
    dx = 50e3
    dom = Domain(p, nx, ny, dx, precision=0)
    assert (dom.nx, dom.ny) == (nx, ny)
    D, eta, R, mask = _case(nx, ny, 11 * nx + ny, even)
    dom.set_fields(D_lith=D, eta_eff=eta, R=R, maskactive=mask)
    spy = dom.scalars()["sec_per_year"]

    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_mask = t(dom.field("maskactive").astype(np.uint8))
    d_D, d_eta = t(dom.field("D_lith")), t(dom.field("eta_eff"))
    d_kap, d_R = t(dom.field("kappa")), t(dom.field("R"))
    stream = torch.cuda.current_stream(dev).cuda_stream

    for call in range(2):                  # two calls in a row through the same scratch
        w, cf = _inputs(nx, ny, 1000 * call + nx)
        want = dom.lvelva(w, cf)
        d_w, d_cf = t(w), t(cf)
        d_out = torch.full((ny, nx), float("nan"), dtype=torch.float64, device=dev)
        rc = L.fi_lvelva_static(d_w.data_ptr(), d_cf.data_ptr(), d_mask.data_ptr(), d_D.data_ptr(),
                                d_eta.data_ptr(), d_kap.data_ptr(), d_R.data_ptr(), nx, ny, dx, dx, p["g"],
                                p["nu"], spy, d_out.data_ptr(), stream)
        assert rc == _lib.FI_OK
        torch.cuda.synchronize(dev)
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, want) <= TOL64, (call, rel(got, want))
    dom.close()


def test_lvelva_static_refuses_oversize():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n = _lib.FI_STATIC_MAX_N + 2
    buf = torch.zeros(n * n, dtype=torch.float64, device="cuda:0")
    m = torch.zeros(n * n, dtype=torch.uint8, device="cuda:0")
    ptr = buf.data_ptr()
    for nx, ny in ((n, 64), (64, n), (63, 64)):
        rc = L.fi_lvelva_static(ptr, ptr, m.data_ptr(), ptr, ptr, ptr, ptr, nx, ny, 50e3, 50e3, 9.81, 0.28,
                                3.15576e7, ptr, None)
        assert rc == _lib.FI_E_SIZE
    torch.cuda.synchronize()
