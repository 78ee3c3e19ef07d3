"""Oracle pins at the benchmark sizes.

The 512^2 headline workload that bench.py times, in both forms: the FP64
kernel-sequence graph (every floating field within 1e-10 of max|value|,
masks bit-exact) and the mixed form through the production step engine and
through the kernel sequence that replaces it on larger grids (displacement
within 1e-5 of max|u| of the FP64 oracle); configuration 1 at
128^2 (reference-compatible Tsit5), configuration 2 at 256^2 (RK4, true
stages) and configuration 3 at 512 x 1024 (interactive sea level, two-layer
freqdomain mantle, reference-compatible Tsit5: the same accept/reject
sequence and bit-exact masks).

The oracle runs on every host core and evaluates the frozen right-hand side
of the reference's stages once per attempt (bit-identical to evaluating it
six times, src/fastisostasy.f90:677-729 ignores the stage state).
"""
import os

import numpy as np
import pytest

from fastisostasy_gb300 import _lib
from fastisostasy_gb300 import workloads as W
from fastisostasy_gb300.isostasy import Domain
from harness import Pair, gpu_bsl, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL64 = 1e-10
TOLMIX = 1e-5
FIELDS = ["w", "we", "z_bed", "dz_ss", "dwdt", "canom_full", "z_ss", "Haf", "x"]
MASKS = ["maskocean", "maskgrounded", "maskcontinent"]


@pytest.fixture(scope="module", autouse=True)
def fast_oracle():
    O.set_threads(os.cpu_count() or 1)
    O.set_reuse_frozen(True)
    yield
    O.set_reuse_frozen(False)


def headline(stage_mode=1):
    """The bench workload: 512^2 at 11.72 km, Gaussian-thinned lithosphere,
    disc load, elastic + geoid, RK4 true stages at dt = 1 yr, dtt = 10 yr."""
    return W.config2(n=512, L=512 * 11.71875e3, dt=1.0, dtt=10.0, stage_mode=stage_mode)


def check_masks(pair):
    """Masks bit-exact, except at ties: cells where the bed and the sea
    surface agree to rounding (|z_bed - z_ss| at 1e-10 of the deflection
    scale), whose comparison z_bed > z_ss (src/sealevel.f90:147-187) any
    rounding decides.  Configuration 1 has such a grid: a flat bed at 0 m
    under a sea surface at 0 m, so its corner cells, where the corner
    boundary condition leaves w at rounding level, are ties."""
    zb, zs = pair.orc.field("z_bed"), pair.orc.field("z_ss")
    scale = max(np.abs(pair.orc.field("w")).max(), np.abs(zb - zb.mean()).max(), 1.0)
    tie = np.abs(zb - zs) <= 1e-10 * scale
    for m in MASKS:
        diff = pair.dom.field(m) != pair.orc.field(m)
        assert not (diff & ~tie).any(), (m, int((diff & ~tie).sum()))
    return int(tie.sum())


def check_fp64(pair):
    worst = {}
    for f in FIELDS:
        a, b = pair.dom.field(f), pair.orc.field(f)
        worst[f] = rel(a, b) if np.abs(b).max() > 0 else float(np.abs(a).max())
        assert worst[f] <= TOL64, (f, worst[f])
    check_masks(pair)
    return worst


def check_counts(pair):
    so, sg = pair.orc.scalars(), pair.dom.scalars()
    assert so["n_accept"] == sg["n_accept"] and so["n_reject"] == sg["n_reject"], (so, sg)
    assert so["t"] == sg["t"]


def used_kernels(dom, t, wl, bsl):
    """Kernel groups one further update launches (CUDA-event profile)."""
    import ctypes as C
    L = dom.L
    L.fi_profile(dom.h, -1)
    L.fi_profile(dom.h, 1)
    _lib.load().fi_bsl_update(bsl, t)
    dom.update(wl.H_at(t), t, bsl)
    nk = len(_lib.PROFILE_KERNELS)
    ms = (C.c_double * nk)()
    cnt = (C.c_longlong * nk)()
    L.fi_profile_read(dom.h, ms, cnt, nk)
    L.fi_profile(dom.h, 0)
    return {k for i, k in enumerate(_lib.PROFILE_KERNELS) if cnt[i] > 0}


def test_headline_512_fp64_graph_matches_oracle():
    """FP64 at 512^2 (src/lv_elva.f90:31-126, src/integrators.f90:42-77 with
    true stages): the captured kernel-sequence graph of every update."""
    pair = Pair(headline(), precision=0)
    assert (pair.dom.nx, pair.dom.ny) == (512, 512)
    pair.init()
    pair.step(2)
    check_fp64(pair)
    check_counts(pair)
    assert "engine" not in used_kernels(pair.dom, pair.t + 10.0, pair.wl, pair.bg)
    pair.close()


def test_headline_512_mixed_engine_matches_oracle():
    """The mixed form exactly as bench.py runs it at 512^2 (the cooperative
    RK4 step engine, four-row items, power-of-two transforms) against the
    FP64 oracle: displacement and elastic displacement within 1e-5."""
    pair = Pair(headline(), precision=1)
    pair.init()
    pair.step(3)
    w_g, w_o = pair.dom.field("w"), pair.orc.field("w")
    assert np.abs(w_o).max() > 1.0
    e = rel(w_g, w_o)
    assert e <= TOLMIX, e
    assert rel(pair.dom.field("we"), pair.orc.field("we")) <= TOLMIX
    assert rel(pair.dom.field("z_bed"), pair.orc.field("z_bed")) <= TOLMIX
    for m in MASKS:
        assert np.array_equal(pair.dom.field(m), pair.orc.field(m)), m
    check_counts(pair)
    assert "engine" in used_kernels(pair.dom, pair.t + 10.0, pair.wl, pair.bg)
    pair.close()


def test_headline_512_mixed_kernel_sequence_matches_oracle(monkeypatch):
    """The mixed form through the kernel sequence that runs where the step
    engine does not fit (1024^2 and up): stage states formed from the float
    pair of x inside the column-strip stencil, the pair advanced with the
    FP64 state.  Against the FP64 oracle within 1e-5, and against the
    engine within the mixed-form bound."""
    monkeypatch.setenv("FI_NO_ENGINE", "1")
    pair = Pair(headline(), precision=1)
    pair.init()
    pair.step(3)
    w_g, w_o = pair.dom.field("w"), pair.orc.field("w")
    e = rel(w_g, w_o)
    assert e <= TOLMIX, e
    assert rel(pair.dom.field("z_bed"), pair.orc.field("z_bed")) <= TOLMIX
    for m in MASKS:
        assert np.array_equal(pair.dom.field(m), pair.orc.field(m)), m
    check_counts(pair)
    used = used_kernels(pair.dom, pair.t + 10.0, pair.wl, pair.bg)
    assert "engine" not in used and "flexure" in used and "rk_final" in used
    w_seq = pair.dom.field("w")
    t_end = pair.t + 10.0
    pair.close()
    monkeypatch.delenv("FI_NO_ENGINE")
    wl = headline()
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=1)
    f = wl.padded_fields(dom.nx, dom.ny)
    if f:
        dom.set_fields(**f)
    bg = gpu_bsl(wl.bsl.get("method", 0), wl.bsl.get("bsl_init", 0.0), wl.bsl.get("A_ocean_pd", 3.625e14))
    dom.init_state(wl.z_bed, wl.H_at(0.0), 0.0, bg)
    t = 0.0
    for _ in range(4):
        t += wl.dtt
        _lib.load().fi_bsl_update(bg, t)
        dom.update(wl.H_at(t), t, bg)
    assert t == t_end
    assert rel(dom.field("w"), w_seq) <= 1e-6
    dom.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_config1_128_tsit54_matches_oracle(precision):
    """Configuration 1 at its full size: 128^2 uniform disc, D = 1e25 N m,
    reference-compatible Tsit5 (src/integrators.f90:131-203)."""
    wl = W.config1(128)
    wl.params["stage_mode"] = 0
    pair = Pair(wl, precision=precision)
    pair.init()
    pair.step(6)
    if precision == 0:
        check_fp64(pair)
        check_counts(pair)
    else:
        assert rel(pair.dom.field("w"), pair.orc.field("w")) <= TOLMIX
    pair.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_config2_256_rk4_matches_oracle(precision):
    """Configuration 2 at its full size: 256^2, Gaussian lithosphere, elastic
    + geoid, RK4 with true stages (dt = 1 yr: 10 yr diverges, lambda*dt ~ -18)."""
    pair = Pair(W.config2(n=256), precision=precision)
    assert (pair.dom.nx, pair.dom.ny) == (256, 256)
    pair.init()
    pair.step(3)
    if precision == 0:
        check_fp64(pair)
    else:
        assert rel(pair.dom.field("w"), pair.orc.field("w")) <= TOLMIX
        assert rel(pair.dom.field("we"), pair.orc.field("we")) <= TOLMIX
    pair.close()


def test_config3_512x1024_fp64_matches_oracle():
    """Configuration 3 at its full size (336 x 560 ice grid padded to
    512 x 1024): interactive sea level, two-layer freqdomain mantle (general
    Hartley multiply), elastic + geoid, the reference's Tsit5.

    That integrator rides the explicit stability edge here (frozen RHS: each
    attempt is a forward-Euler step whose error estimate does not see
    stability), so rounding-level differences grow by about 1e4 per model
    year: a 1e-13 change of the upper-mantle viscosity moves the oracle's
    own solution by ~2e-9 of max|w| at t = 2 yr and by ~0.3 at t = 4 yr, with
    a different accept/reject sequence (test_oracle.py pins this on the
    CPU).  The comparison therefore runs over the first two model years
    (about 45 attempts): the same accept/reject sequence, masks bit-exact,
    every field within 1e-10 at t = 1 yr, and at t = 2 yr w closer to the
    oracle than the oracle is to itself under that 1e-13 change."""
    wl = W.config3()
    pair = Pair(wl, precision=0)
    assert (pair.dom.nx, pair.dom.ny) == (512, 1024)
    pair.init()
    for t in (0.5, 1.0):
        pair.wl.dtt = t - pair.t
        pair.step(1)
        check_counts(pair)
    check_fp64(pair)
    assert check_masks(pair) == 0   # a fractal bed: no ties
    assert pair.dom.field("maskocean").any() and pair.dom.field("maskcontinent").any()
    pair.wl.dtt = 1.0
    pair.step(1)                    # t = 2 yr
    check_counts(pair)
    assert pair.orc.scalars()["n_reject"] > 10
    assert check_masks(pair) == 0
    w_g, w_o = pair.dom.field("w"), pair.orc.field("w")
    pair.close()
    wp = W.config3()
    wp.params["viscosities"] = [1e20 * (1 + 1e-13), 1e21]
    m = O.Model(wp.params, wp.nx_ice, wp.ny_ice, wp.dx, wp.dx)
    b = O.make_bsl()
    m.init_state(wp.z_bed, wp.H_at(0.0), 0.0, b)
    for t in (0.5, 1.0, 2.0):
        assert m.update(wp.H_at(t), t, b) == 0
    sens = rel(m.field("w"), w_o)
    m.close()
    assert 1e-12 < sens < 1e-6, sens
    assert rel(w_g, w_o) <= sens, (rel(w_g, w_o), sens)
