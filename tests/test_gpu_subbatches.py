"""hepem_step_subbatches: many sub-batches of one set of arrays, each with its
own RNG key, stepped in one sorted, queued pass, against one
hepem_step_batched / hepem_step_mixed call per sub-batch (bit for bit), with
gaps between sub-batches left untouched, and the argument checks."""
import numpy as np
import pytest

from conftest import T16
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu

NU = 32


@pytest.mark.parametrize("form", ["batched", "mixed"])
@pytest.mark.parametrize("in_place", [False, True])
def test_subbatches_equal_one_call_per_subbatch(native, gpu_ctx, form, in_place):
    import torch
    ctx = gpu_ctx(T16)
    total = 120000
    st = W.mixed_batch(total, n_couples=16, seed=61, emin=1e-3, emax=1e5)
    rng = np.random.default_rng(5)
    # sub-batches of uneven sizes with gaps between some of them, given out of order
    cuts = np.sort(rng.choice(np.arange(1, total), 40, replace=False))
    edges = np.concatenate([[0], cuts, [total]])
    batches = []
    for k in range(len(edges) - 1):
        a, e = int(edges[k]), int(edges[k + 1])
        if k % 7 == 3:
            continue  # a gap
        batches.append((a, e - a, 1000 + 17 * k))
    batches = [batches[i] for i in rng.permutation(len(batches))]
    sin = native.state_to_torch(st)
    u = native.fill_uniforms(sin["id"], NU, 0)  # the buffer is the same for every key here
    res = native.alloc_out_torch(total)
    sentinel = -7.0
    sout = sin if in_place else native.state_to_torch(st)
    if not in_place:
        sout["ekin"].fill_(sentinel)
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step_subbatches(batches, sin, sout, u, NU, res, counters=cnt, form=form)
    torch.cuda.synchronize()
    got, got_res = native.to_numpy(sout), native.to_numpy(res)
    slots = {f: k for f, _, k in native.OUT_FIELDS}
    covered = np.zeros(total, bool)
    steps = 0
    for a, n, seed in batches:
        e = a + n
        covered[a:e] = True
        steps += n
        s1 = native.state_to_torch({k: v[a:e] for k, v in st.items()})
        o1 = native.empty_state_torch(n)
        r1 = native.alloc_out_torch(n)
        ctx.step(s1, o1, u[a * NU:e * NU], NU, seed, r1, form=form)
        torch.cuda.synchronize()
        o1, r1 = native.to_numpy(o1), native.to_numpy(r1)
        for k in native.STATE_OUT_FIELDS:
            assert np.array_equal(got[k][a:e], o1[k], equal_nan=True), (a, k)
        for k, v in r1.items():
            m = slots[k]
            assert np.array_equal(got_res[k][a * m:e * m], v, equal_nan=True), (a, k)
    # tracks outside every sub-batch are left untouched
    if in_place:
        assert np.array_equal(got["ekin"][~covered], st["ekin"][~covered])
    else:
        assert np.all(got["ekin"][~covered] == sentinel)
    assert int(cnt[0].item()) == steps


@pytest.mark.parametrize("form", ["batched", "mixed"])
def test_subbatches_without_uniforms(native, gpu_ctx, form):
    """n_uniform = 0 over more than 2^20 tracks: the library draws the first
    values of every stream ahead (one row per stepped track, found through the
    active list) and the rest in place; the results equal a step of each
    sub-batch alone, which draws every value in place (the FP64 form: the
    plain form's), bit for bit, the flag of draws past the (empty) buffer
    included."""
    import torch
    ctx = gpu_ctx(T16)
    # more than 2^20 tracks stepped: the library draws ahead (smaller batches draw in place)
    total = (1 << 20) + 60000
    st = W.mixed_batch(total, n_couples=16, seed=62, emin=1e-3, emax=1e5)
    batches = [(0, 500000, 11), (520000, 300000, 12), (830000, total - 830000, 13)]
    sin = native.state_to_torch(st)
    sout = native.state_to_torch(st)
    res = native.alloc_out_torch(total)
    ctx.step_subbatches(batches, sin, sout, None, 0, res, form=form)
    torch.cuda.synchronize()
    got, got_res = native.to_numpy(sout), native.to_numpy(res)
    slots = {f: k for f, _, k in native.OUT_FIELDS}
    drawn = []
    for a, n, seed in batches:
        e = a + n
        s1 = native.state_to_torch({k: v[a:e] for k, v in st.items()})
        o1 = native.empty_state_torch(n)
        r1 = native.alloc_out_torch(n)
        ctx.step(s1, o1, None, 0, seed, r1, form="plain" if form == "batched" else form)
        torch.cuda.synchronize()
        o1, r1 = native.to_numpy(o1), native.to_numpy(r1)
        for k in native.STATE_OUT_FIELDS:
            assert np.array_equal(got[k][a:e], o1[k], equal_nan=True), (a, k)
        for k, v in r1.items():
            m = slots[k]
            assert np.array_equal(got_res[k][a * m:e * m], v, equal_nan=True), (a, k)
        drawn.append(o1["rng_cursor"] - st["rng_cursor"][a:e])
    drawn = np.concatenate(drawn)
    # some tracks drew past the values drawn ahead (32), every drawing track raised the flag
    assert drawn.max() > 32
    flags = np.concatenate([got_res["flags"][a:a + n] for a, n, _ in batches])
    assert np.array_equal(flags & 1, (drawn > 0).astype(np.uint8))


@pytest.mark.parametrize("form", ["batched", "mixed"])
def test_large_step_without_uniforms(native, gpu_ctx, form):
    """n_uniform = 0 over more than 2^20 tracks in one dense call: equal, bit
    for bit, to the same tracks stepped in two calls below 2^20 tracks (which
    draw in place), and for the FP64 form to the plain form."""
    import torch
    ctx = gpu_ctx(T16)
    n = (1 << 20) + 4096
    st = W.mixed_batch(n, n_couples=16, seed=63, emin=1e-3, emax=1e5)
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    ctx.step(sin, sout, None, 0, 77, res, form=form)
    torch.cuda.synchronize()
    got, got_res = native.to_numpy(sout), native.to_numpy(res)
    slots = {f: k for f, _, k in native.OUT_FIELDS}
    for a, e in ((0, n // 2), (n // 2, n)):
        m = e - a
        s1 = native.state_to_torch({k: v[a:e] for k, v in st.items()})
        o1 = native.empty_state_torch(m)
        r1 = native.alloc_out_torch(m)
        ctx.step(s1, o1, None, 0, 77, r1, form="plain" if form == "batched" else form)
        torch.cuda.synchronize()
        o1, r1 = native.to_numpy(o1), native.to_numpy(r1)
        for k in native.STATE_OUT_FIELDS:
            assert np.array_equal(got[k][a:e], o1[k], equal_nan=True), (a, k)
        for k, v in r1.items():
            q = slots[k]
            assert np.array_equal(got_res[k][a * q:e * q], v, equal_nan=True), (a, k)


def test_subbatches_reject_overlaps_and_bad_forms(native, gpu_ctx):
    ctx = gpu_ctx(T16)
    st = native.state_to_torch(W.mixed_batch(1000, n_couples=16, seed=3))
    res = native.alloc_out_torch(1000)
    out = native.empty_state_torch(1000)
    with pytest.raises(native.HepEmError) as e:
        ctx.step_subbatches([(0, 600, 1), (500, 400, 2)], st, out, None, 0, res)
    assert "overlap" in str(e.value)
    with pytest.raises(native.HepEmError):
        ctx.step_subbatches([(0, 10, 1)], st, out, None, 0, res, form="plain")
    with pytest.raises(native.HepEmError):
        ctx.step_subbatches([(-1, 10, 1)], st, out, None, 0, res)
    ctx.step_subbatches([], st, out, None, 0, res)  # nothing to do
