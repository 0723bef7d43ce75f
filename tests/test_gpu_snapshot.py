"""Server snapshot and resume (hepem_server_snapshot / hepem_server_resume):
requests snapshotted mid-run -- some resident with steps taken, some still
waiting for memory -- and resumed on a fresh server end with the results and
final track state of the uninterrupted run, bit for bit, in both precisions."""
import time

import numpy as np
import pytest

from conftest import T3
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu

MIN_E = 1.0e-3


def _server(native, ctx, mixed, budget=48 << 20):
    return native.Server(ctx, memory_budget_bytes=budget, max_steps=150, min_energy=MIN_E, mixed=mixed)


@pytest.mark.parametrize("mixed", [False, True])
def test_resume_equals_uninterrupted(native, gpu_ctx, mixed):
    ctx = gpu_ctx(T3)
    a = _server(native, ctx, mixed)
    b = None
    try:
        n = a.capacity * 2 // 5          # two requests resident at once, the rest wait
        reqs = [W.mixed_batch(n, n_couples=3, seed=40 + k, emin=1.0, emax=1.0e4) for k in range(5)]
        ids = [a.submit(r, seed=500 + k) for k, r in enumerate(reqs)]
        t0 = time.time()
        while a.stats()["iterations"] < 6 and time.time() - t0 < 60:
            time.sleep(0.002)
        snap = a.snapshot()
        full = {rid: a.wait(rid, want_tracks=True) for rid in ids}
        recs = native.snapshot_records(snap)
        assert native.snapshot_check(snap) == (len(recs), sum(r["n"] for r in recs))
        assert any(r["admitted"] and r["steps"] > 0 for r in recs), [(r["id"], r["steps"]) for r in recs]
        assert any(not r["admitted"] for r in recs)
        b = _server(native, ctx, mixed)
        mapping = b.resume(snap)
        assert sorted(mapping) == [r["id"] for r in recs]
        for old, new in mapping.items():
            res_b, fin_b = b.wait(new, want_tracks=True)
            res_a, fin_a = full[old]
            for k in ("n_tracks", "steps", "status", "edep", "e_secondaries", "n_secondaries", "track_steps"):
                assert res_a[k] == res_b[k], (old, k, res_a[k], res_b[k])
            for k in fin_a:
                assert np.array_equal(fin_a[k], fin_b[k]), (old, k)
    finally:
        a.close()
        if b is not None:
            b.close()


def test_snapshot_of_idle_server_and_bad_resume(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    a = _server(native, ctx, False)
    b = _server(native, ctx, False, budget=8 << 20)
    try:
        snap = a.snapshot()
        assert native.snapshot_check(snap) == (0, 0)
        assert b.resume(snap) == {}
        # a request larger than the resuming server's pool: refused, nothing submitted
        rid = a.submit(W.mixed_batch(b.capacity + 1000, n_couples=3, seed=3), seed=1)
        snap = a.snapshot()
        with pytest.raises(native.HepEmError) as e:
            b.resume(snap)
        assert e.value.code == native.STATUS_OOM_ADMISSION
        assert b.stats()["waiting"] == 0 and b.stats()["active"] == 0
        a.wait(rid)
    finally:
        a.close()
        b.close()
