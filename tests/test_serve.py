"""Solve server (fi_serve_*): results against directly driven handles, the
same request alone and in a mix, admission limits, ensembles."""
import numpy as np
import pytest

from fastisostasy_gb300 import workloads as W
from fastisostasy_gb300.isostasy import Domain
from fastisostasy_gb300.serve import Server, padded_dims
from harness import gpu_bsl, mixed_bound, oracle_solve, rel
from fastisostasy_gb300 import _lib
from oracle import oracle as O


def small_rk4(n=48, seed=0, stage_mode=1):
    wl = W.config2(n=n, L=3000e3 * n / 256, dt=1.0, stage_mode=stage_mode)
    wl.t_end = 60.0
    return wl


def small_tsit(n=40):
    wl = W.config1(n)
    wl.params["stage_mode"] = 0
    wl.t_end = 50.0
    return wl


def direct(wl, precision=0):
    """The same solve through one handle driven by isos_update calls."""
    dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
    f = wl.padded_fields(dom.nx, dom.ny)
    if f:
        dom.set_fields(**f)
    b = gpu_bsl()
    dom.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
    out = {"w": np.zeros((wl.ny_ice, wl.nx_ice)), "z_bed": np.zeros((wl.ny_ice, wl.nx_ice))}
    t = 0.0
    while t < wl.t_end:
        t = min(t + wl.dtt, wl.t_end)
        dom.update(wl.H_final, t, b, out=out)
    dom.close()
    return out["w"], out["z_bed"]


def test_padded_dims_match_oracle():
    """fi_padded_dims (no device needed) against the oracle's domain."""
    for wl in (small_rk4(48), small_tsit(40), W.config3(nx_ice=40, ny_ice=72, dx=20e3, nx_pad=64, ny_pad=96)):
        m = O.Model(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, wl.dx)
        nx, ny = padded_dims(wl.params, wl.nx_ice, wl.ny_ice, wl.dx)[:2]
        assert (nx, ny) == (m.nx, m.ny)
        m.close()


@pytest.mark.gpu
@pytest.mark.parametrize("make,precision", [(small_rk4, 0), (small_rk4, 1), (small_tsit, 0)])
def test_served_solve_matches_direct_handle(make, precision):
    wl = make()
    w_ref, zb_ref = direct(wl, precision)
    srv = Server(max_inflight=4, reserve_gb=1.0)
    rid = srv.submit(wl, precision=precision)
    info = srv.wait(rid, 120.0)
    assert info["state"] == "done" and info["status"] == 0
    w, zb = srv.result(rid)
    srv.close()
    assert np.array_equal(w, w_ref) and np.array_equal(zb, zb_ref)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_alone_and_in_a_mix_are_identical(precision):
    """Continuous batching: a request gives the same bits alone and while
    requests of other sizes and integrators run beside it."""
    target = small_rk4(64)
    srv = Server(max_inflight=16, reserve_gb=1.0)
    rid = srv.submit(target, precision=precision)
    srv.wait(rid, 120.0)
    alone = srv.result(rid)
    others = []
    for i, n in enumerate((32, 48, 96, 128, 40, 80)):
        others.append(srv.submit(small_rk4(n), precision=precision))
        if i == 2:
            rid = srv.submit(target, precision=precision)   # arrives while others run
        others.append(srv.submit(small_tsit(32 + 8 * (i % 3)), precision=0))
    info = srv.wait(rid, 300.0)
    assert info["status"] == 0, info
    mixed = srv.result(rid)
    for o in others:
        io = srv.wait(o, 300.0)
        assert io["status"] == 0, io
        srv.result(o)
    srv.close()
    assert np.array_equal(alone[0], mixed[0]) and np.array_equal(alone[1], mixed[1])


@pytest.mark.gpu
def test_every_request_of_a_repeated_mix_matches_its_solve_alone():
    """Regression for a load upload that was not ordered before the handle's
    stream: run the same mix of mixed-form step-engine requests (and FP64
    Tsit5 ones beside them) several times and compare every request, not one,
    with its solve alone."""
    sizes = (32, 48, 96, 128, 40, 80, 64)
    srv = Server(max_inflight=1, reserve_gb=1.0)
    alone = {}
    for n in sizes:
        rid = srv.submit(small_rk4(n), precision=1)
        srv.wait(rid, 120.0)
        alone[n] = srv.result(rid)
    srv.close()
    for _ in range(12):
        srv = Server(max_inflight=16, reserve_gb=1.0)
        ids = []
        for i, n in enumerate(sizes[:6]):
            ids.append((n, srv.submit(small_rk4(n), precision=1)))
            if i == 2:
                ids.append((64, srv.submit(small_rk4(64), precision=1)))
            ids.append((None, srv.submit(small_tsit(32 + 8 * (i % 3)), precision=0)))
        for n, rid in ids:
            info = srv.wait(rid, 300.0)
            assert info["status"] == 0, info
            w, zb = srv.result(rid)
            if n is not None:
                assert np.array_equal(w, alone[n][0]) and np.array_equal(zb, alone[n][1]), n
        srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_served_requests_match_oracle(precision):
    """Two requests of different sizes and integrators served side by side,
    each against the oracle: FP64 within 1e-10, mixed within 1e-5."""
    wls = [small_rk4(48), small_tsit(40)]
    srv = Server(max_inflight=4, reserve_gb=1.0)
    ids = [srv.submit(wl, precision=precision) for wl in wls]
    res = []
    for rid in ids:
        info = srv.wait(rid, 120.0)
        assert info["status"] == 0, info
        res.append(srv.result(rid)[0])
    srv.close()
    for wl, w in zip(wls, res):
        times = [min(wl.dtt * (k + 1), wl.t_end) for k in range(int(np.ceil(wl.t_end / wl.dtt)))]
        wo = oracle_solve(wl, times)
        dom_pd = padded_dims(wl.params, wl.nx_ice, wl.ny_ice, wl.dx)
        i1, i2, j1, j2 = dom_pd[2:]
        wo = wo[j1 - 1:j2, i1 - 1:i2]
        assert rel(w, wo) <= (1e-10 if precision == 0 else 1e-5)


@pytest.mark.gpu
def test_cancel_running_and_queued_requests():
    """fi_serve_cancel: a running request stops issuing updates and is
    retired; a queued one never starts; the requests beside them finish with
    the bits they get alone."""
    long_wl = small_rk4(96)
    long_wl.t_end = 20000.0           # 2000 updates: still running when cancelled
    nb = [small_rk4(48), small_tsit(40)]
    want = [direct(wl) for wl in nb]
    srv = Server(max_inflight=8, reserve_gb=1.0)
    rl = srv.submit(long_wl)
    ids = [srv.submit(wl) for wl in nb]
    import time
    t0 = time.time()
    while srv.info(rl)["updates"] < 4:
        assert time.time() - t0 < 60.0
        time.sleep(0.002)
    srv.cancel(rl)
    info = srv.wait(rl, 60.0)
    assert info["state"] == "cancelled" and info["status"] == _lib.FI_E_CANCELLED
    assert 4 <= info["updates"] < 2000
    with pytest.raises(_lib.FiError) as e:
        srv.result(rl)
    assert e.value.code == _lib.FI_E_CANCELLED
    for rid, (w_ref, zb_ref) in zip(ids, want):
        assert srv.wait(rid, 120.0)["state"] == "done"
        w, zb = srv.result(rid)
        assert np.array_equal(w, w_ref) and np.array_equal(zb, zb_ref)
    with pytest.raises(_lib.FiError) as e:
        srv.cancel(rl)               # released
    srv.close()
    # a queued request: one slot, held by a long solve
    srv = Server(max_inflight=1, reserve_gb=1.0)
    ra = srv.submit(long_wl)
    rb = srv.submit(small_rk4(48))
    assert srv.info(rb)["state"] == "queued"
    srv.cancel(rb)
    ib = srv.wait(rb, 10.0)
    assert ib["state"] == "cancelled" and ib["updates"] == 0
    srv.cancel(ra)
    assert srv.wait(ra, 60.0)["state"] == "cancelled"
    srv.close()


@pytest.mark.gpu
def test_request_that_cannot_fit_fails_with_oom():
    """Admission by device memory: with a reserve larger than the device, no
    request can ever be admitted, and each fails at once with FI_E_OOM
    instead of waiting; a server with room still solves the same request."""
    wl = small_rk4(48)
    srv = Server(max_inflight=4, reserve_gb=1e6)
    ids = [srv.submit(wl) for _ in range(2)]
    for rid in ids:
        info = srv.wait(rid, 30.0)
        assert info["state"] == "failed" and info["status"] == _lib.FI_E_OOM, info
        assert "device has" in info["error"]
        with pytest.raises(_lib.FiError):
            srv.result(rid)
    srv.close()
    srv = Server(max_inflight=4, reserve_gb=1.0)
    rid = srv.submit(wl)
    assert srv.wait(rid, 120.0)["state"] == "done"
    w, _ = srv.result(rid)
    srv.close()
    assert np.array_equal(w, direct(wl)[0])


@pytest.mark.gpu
def test_inflight_cap_and_drain():
    srv = Server(max_inflight=2, reserve_gb=0.5)
    ids = [srv.submit(small_rk4(48)) for _ in range(5)]
    infos = [srv.wait(i, 300.0) for i in ids]
    assert all(i["state"] == "done" for i in infos)
    for k in range(2, 5):
        # at most two run at once: the k-th starts after the (k-2)-th ended
        done = sorted(i["t_done"] for i in infos[:k])
        assert infos[k]["t_admit"] >= done[k - 2] - 1e-6
    for i in ids:
        srv.result(i)
    srv.close()


@pytest.mark.gpu
def test_unstable_request_fails_alone():
    """A request whose solve diverges reports FI_E_LARGE; its neighbours finish."""
    bad = W.config2(n=64, L=3000e3 * 64 / 256 * 2, dt=50.0, stage_mode=1)
    bad.t_end = 2000.0
    bad.dtt = 100.0
    good = small_rk4(48)
    srv = Server(max_inflight=4, reserve_gb=0.5)
    rb, rg = srv.submit(bad), srv.submit(good)
    ib, ig = srv.wait(rb, 120.0), srv.wait(rg, 120.0)
    srv.close()
    assert ib["state"] == "failed" and ib["status"] in (1, 2)
    assert ig["state"] == "done"


def ens_members(mode):
    if mode == "streams":
        return [small_rk4(48), small_tsit(40), small_rk4(64), small_tsit(56)]
    # batched launches: reference-compatible Tsit5 members of different sizes
    # and rheologies
    out = [small_tsit(40), small_tsit(56)]
    for i in (3, 7):
        wl = W.ensemble_member(i, stage_mode=0)
        out.append(wl)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision,mode", [(0, "streams"), (1, "streams"), (0, "graph"), (1, "graph")])
def test_ensemble_lockstep_matches_members_alone(precision, mode):
    """Lockstep ensembles (per-member streams, or one graph of batched
    launches) give each member the bits it gets when driven alone."""
    from fastisostasy_gb300.serve import Ensemble
    wls = ens_members(mode)
    ens = Ensemble(wls, precision=precision, mode=mode)
    ens.first_update(10.0)
    for t in (20.0, 30.0, 40.0, 50.0, 60.0):
        ens.update(t)
    ens.synchronize()
    got = [d.field("w") for d in ens.doms]
    counts = {}
    for wl, d in zip(wls, ens.doms):
        sc = d.scalars()
        counts[wl.name] = (sc["n_accept"], sc["n_reject"])
    ens.close()
    for wl, g in zip(wls, got):
        wl.t_end = 60.0
        dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
        f = wl.padded_fields(dom.nx, dom.ny)
        if f:
            dom.set_fields(**f)
        b = gpu_bsl()
        dom.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        for t in (10.0, 20.0, 30.0, 40.0, 50.0, 60.0):
            dom.update(wl.H_final, t, b)
        w = dom.field("w")
        dom.close()
        if mode == "graph" and wl.name.startswith("member_"):
            # the batched member against the oracle as well
            times = (10.0, 20.0, 30.0, 40.0, 50.0, 60.0)
            wo, co = oracle_solve(wl, times, counts=True)
            if precision == 0:
                assert counts[wl.name] == co
            bound = 1e-10 if precision == 0 else mixed_bound(wl, times, wo)[0]
            assert rel(g, wo) <= bound, (wl.name, rel(g, wo), bound, counts[wl.name], co)
        if mode == "graph" and precision == 1:
            # the batched launches are other kernels built from the same
            # code; the compiler may fuse FP32 multiply-adds differently in
            # them (with contraction off the two agree bit for bit), and the
            # adaptive steps carry those roundings on: the mixed form's bound
            assert np.abs(w - g).max() <= 1e-5 * np.abs(w).max()
        else:
            assert np.array_equal(w, g)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_true_stage_ensemble_matches_members_alone(precision):
    """Batched Tsit5 with true stages (Dormand-Prince 5(4), FSAL) over
    members of different sizes: each member's result equals driving it
    alone (FP64 bit for bit; mixed to the mixed-form bound)."""
    from fastisostasy_gb300.serve import Ensemble
    wls = []
    for wl in (small_tsit(40), small_tsit(56), W.ensemble_member(3, stage_mode=1), W.ensemble_member(7, stage_mode=1)):
        wl.params["stage_mode"] = 1
        wls.append(wl)
    ens = Ensemble(wls, precision=precision, mode="graph")
    ens.first_update(10.0)
    for t in (20.0, 30.0, 40.0, 50.0):
        ens.update(t)
    ens.synchronize()
    got = [d.field("w") for d in ens.doms]
    ens.close()
    for wl, g in zip(wls, got):
        dom = Domain(wl.params, wl.nx_ice, wl.ny_ice, wl.dx, precision=precision)
        f = wl.padded_fields(dom.nx, dom.ny)
        if f:
            dom.set_fields(**f)
        b = gpu_bsl()
        dom.init_state(wl.z_bed, np.zeros_like(wl.H_final), 0.0, b)
        for t in (10.0, 20.0, 30.0, 40.0, 50.0):
            dom.update(wl.H_final, t, b)
        w = dom.field("w")
        dom.close()
        if precision == 1:
            # the batched launches are other kernels built from the same
            # code (the compiler may fuse FP32 multiply-adds differently);
            # the members of configuration 4 amplify such roundings in their
            # stiff modes, so their bound is the mixed form's against the
            # oracle: ten times the oracle's own move under FP32-sized noise
            bound = 1e-5
            if wl.name.startswith("member_"):
                times = (10.0, 20.0, 30.0, 40.0, 50.0)
                bound = mixed_bound(wl, times, oracle_solve(wl, times))[0]
            assert np.abs(w - g).max() <= bound * np.abs(w).max(), (wl.name, rel(g, w), bound)
        else:
            assert np.array_equal(w, g)
