"""Serving form (hepem_server_*): continuous batching of event requests.

A request's result must not depend on what else is resident: each track draws
pure Philox uniforms keyed by the request seed and its own id, and the
per-request sums are reduced in a fixed order.  The results are also checked
against the CPU port stepped the same way (tracks above min_energy step once
per iteration, until none is left or the step budget is used up).
"""
import numpy as np
import pytest

from conftest import T3, T16
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu

MIN_E = 1.0e-3  # MeV: tracks below 1 keV leave the server


def port_serve(port_lib, tracks, seed, max_steps, min_e=MIN_E):
    """The serving loop of one request on the CPU port: every iteration steps
    the tracks with ekin > min_e (nu = 0: pure Philox streams).  Returns the
    final state, per-track sums (edep, secondary energy, secondaries, steps)
    and the number of iterations that stepped something."""
    st = {k: np.array(v, copy=True) for k, v in tracks.items()}
    n = len(st["ekin"])
    edep = np.zeros(n)
    esec = np.zeros(n)
    nsec = np.zeros(n, dtype=np.int64)
    tsteps = np.zeros(n, dtype=np.int64)
    it = 0
    while it < max_steps:
        alive = np.nonzero(st["ekin"] > min_e)[0]
        if len(alive) == 0:
            break
        sub = {k: np.ascontiguousarray(v[alive]) for k, v in st.items()}
        out, res = port_lib.step(sub, np.zeros(0), 0, seed)
        for k in st:
            st[k][alive] = out[k]
        edep[alive] += res["edep"]
        ns = res["n_sec"].astype(np.int64)
        se = res["sec_ekin"].reshape(-1, 2)
        esec[alive] += np.where(ns > 0, se[:, 0], 0.0) + np.where(ns > 1, se[:, 1], 0.0)
        nsec[alive] += ns
        tsteps[alive] += 1
        it += 1
    return st, dict(edep=edep, esec=esec, nsec=nsec, tsteps=tsteps), it


def _request(n, seed, id0=0, emin=1.0, emax=1.0e4, nc=3):
    return W.mixed_batch(n, n_couples=nc, seed=seed, emin=emin, emax=emax, id0=id0)


def _same_result(a, b):
    for k in ("n_tracks", "steps", "status", "edep", "e_secondaries", "n_secondaries", "track_steps"):
        assert a[k] == b[k], (k, a[k], b[k])


def _same_tracks(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_server_request_matches_port(native, gpu_ctx, port):
    ctx = gpu_ctx(T3)
    srv = native.Server(ctx, memory_budget_bytes=64 << 20, max_steps=30, min_energy=MIN_E)
    try:
        req = _request(2000, seed=21)
        rid = srv.submit(req, seed=99)
        res, fin = srv.wait(rid, want_tracks=True)
    finally:
        srv.close()
    st, sums, it = port_serve(port(T3), req, 99, 30)
    assert res["status"] == 0
    assert res["steps"] == it
    assert res["n_secondaries"] == sums["nsec"].sum()
    assert res["track_steps"] == sums["tsteps"].sum()
    # per-request sums: fixed-order tree on the device, sequential here (1e-12 relative)
    assert res["edep"] == pytest.approx(sums["edep"].sum(), rel=1e-12)
    assert res["e_secondaries"] == pytest.approx(sums["esec"].sum(), rel=1e-12)
    # per-track state after `it` steps: energies and the RNG position exactly, directions to 1e-12
    for k in ("ekin", "rng_cursor", "gauss_valid", "msc_first_step", "nia0", "nia1", "nia2", "nia3"):
        np.testing.assert_allclose(fin[k], st[k], rtol=1e-12, atol=0, err_msg=k)
    for k in ("dir_x", "dir_y", "dir_z"):
        np.testing.assert_allclose(fin[k], st[k], rtol=0, atol=1e-12, err_msg=k)


def test_server_runs_requests_to_completion(native, gpu_ctx, port):
    # 1-10 MeV tracks end below 1 keV well within the step budget
    ctx = gpu_ctx(T3)
    srv = native.Server(ctx, memory_budget_bytes=64 << 20, max_steps=5000, min_energy=MIN_E)
    try:
        req = _request(600, seed=4, emin=1.0, emax=10.0)
        res, fin = srv.wait(srv.submit(req, seed=5), want_tracks=True)
    finally:
        srv.close()
    st, sums, it = port_serve(port(T3), req, 5, 5000)
    assert it < 5000 and res["steps"] == it
    assert np.all(fin["ekin"] <= MIN_E)
    assert res["track_steps"] == sums["tsteps"].sum()
    assert res["edep"] == pytest.approx(sums["edep"].sum(), rel=1e-12)


def test_server_result_same_alone_and_in_the_mix(native, gpu_ctx):
    ctx = gpu_ctx(T16)
    srv = native.Server(ctx, memory_budget_bytes=256 << 20, max_steps=40, min_energy=MIN_E)
    try:
        a = _request(3000, seed=5, nc=16)
        alone, fin_alone = srv.wait(srv.submit(a, seed=77), want_tracks=True)
        others = [_request(m, seed=s, id0=0, nc=16) for m, s in ((5000, 6), (700, 8), (12000, 9), (64, 10))]
        ids = [srv.submit(others[0], seed=1), srv.submit(others[1], seed=2)]
        ra = srv.submit(a, seed=77)
        ids += [srv.submit(others[2], seed=3), srv.submit(others[3], seed=4)]
        mixed, fin_mixed = srv.wait(ra, want_tracks=True)
        rest = [srv.wait(i)[0] for i in ids]
    finally:
        srv.close()
    _same_result(alone, mixed)
    _same_tracks(fin_alone, fin_mixed)
    # the requests were resident together: every admission came before any completion
    allr = rest + [mixed]
    assert max(r["t_admit"] for r in allr) < min(r["t_done"] for r in allr)
    assert all(r["status"] == 0 for r in allr)


def test_server_admission_by_memory_budget(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    srv = native.Server(ctx, memory_budget_bytes=8 << 20, max_steps=6, min_energy=MIN_E)
    try:
        cap = srv.capacity
        assert 10000 < cap < 40000
        with pytest.raises(native.HepEmError) as e:
            srv.submit(_request(cap + 1, seed=1), seed=1)
        assert e.value.code == native.STATUS_OOM_ADMISSION
        m = cap // 3 + 1                       # at most two of these fit at once
        reqs = [_request(m, seed=30 + k) for k in range(6)]
        ids = [srv.submit(r, seed=k) for k, r in enumerate(reqs)]
        res = [srv.wait(i)[0] for i in ids]
        # each one alone gives the same result
        solo = [srv.wait(srv.submit(r, seed=k))[0] for k, r in enumerate(reqs)]
        st = srv.stats()
    finally:
        srv.close()
    for r, s in zip(res, solo):
        _same_result(r, s)
    admits = [r["t_admit"] for r in res]
    assert admits == sorted(admits)             # first come, first served
    # at most two resident at a time: the third waited for the first to finish
    assert res[2]["t_admit"] >= min(res[0]["t_done"], res[1]["t_done"])
    assert st["free_slots"] == cap and st["active"] == 0 and st["waiting"] == 0


def test_server_cancel_and_bounded_wait(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    srv = native.Server(ctx, memory_budget_bytes=64 << 20, max_steps=1000000, min_energy=MIN_E)
    try:
        cap = srv.capacity
        big = _request(cap - 10, seed=3, emin=1.0e3, emax=1.0e4)
        rb = srv.submit(big, seed=1)
        rw = srv.submit(_request(100, seed=4), seed=2)   # cannot be admitted while `big` runs
        with pytest.raises(native.HepEmError) as e:
            srv.wait(rb, timeout_s=0.0)
        assert e.value.code == native.STATUS_TIMEOUT
        srv.cancel(rw)
        res_w, _ = srv.wait(rw, timeout_s=30.0)
        assert res_w["status"] == native.STATUS_CANCELLED and res_w["steps"] == 0
        srv.cancel(rb)                               # hundreds of steps from done
        res_b, fin_b = srv.wait(rb, timeout_s=60.0, want_tracks=True)
        assert res_b["status"] == native.STATUS_CANCELLED
        assert np.all(np.isfinite(fin_b["ekin"]))
        # the server keeps serving after cancellations
        r, _ = srv.wait(srv.submit(_request(500, seed=9), seed=3), timeout_s=60.0)
        assert r["status"] == 0
        with pytest.raises(native.HepEmError):
            srv.wait(12345678, timeout_s=0.1)       # unknown request id
    finally:
        srv.close()


def test_server_precision_form(native, gpu_ctx):
    # The serving loop over the precision form: results are independent of
    # the mix.  Against the FP64 server: one iteration gives the same discrete
    # history (step and secondary counts) and sums within 1e-5.  Over many
    # iterations the two trajectories start from states that differ by the
    # FP32 rounding of the previous steps, so only the totals are compared.
    ctx = gpu_ctx(T3)
    a = _request(4000, seed=14)
    res = {}
    for mixed in (False, True):
        for steps in (1, 50):
            srv = native.Server(ctx, memory_budget_bytes=128 << 20, max_steps=steps, min_energy=MIN_E,
                                mixed=mixed)
            try:
                alone, fin_alone = srv.wait(srv.submit(a, seed=5), want_tracks=True)
                ids = [srv.submit(_request(3000, seed=s), seed=s) for s in (31, 32)]
                ra = srv.submit(a, seed=5)
                ids.append(srv.submit(_request(9000, seed=33), seed=33))
                mix, fin_mix = srv.wait(ra, want_tracks=True)
                for i in ids:
                    srv.wait(i)
            finally:
                srv.close()
            _same_result(alone, mix)
            _same_tracks(fin_alone, fin_mix)
            res[(mixed, steps)] = alone
    f64, f32 = res[(False, 1)], res[(True, 1)]
    for k in ("steps", "n_secondaries", "track_steps", "status"):
        assert f64[k] == f32[k], k
    assert f32["edep"] == pytest.approx(f64["edep"], rel=1e-5)
    assert f32["e_secondaries"] == pytest.approx(f64["e_secondaries"], rel=1e-5)
    f64, f32 = res[(False, 50)], res[(True, 50)]
    assert f32["edep"] == pytest.approx(f64["edep"], rel=2e-2)
    assert f32["n_secondaries"] == pytest.approx(f64["n_secondaries"], rel=2e-2)
