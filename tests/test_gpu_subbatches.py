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
