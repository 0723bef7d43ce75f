"""Several host threads stepping on one context at once, each on its own
stream: the batched steps fork their independent stages onto the context's
side streams and join them back, with the enqueue of each step's forks and
joins under one lock.  Every thread's results must equal the same steps made
one after another on one stream, bit for bit, in both batched forms."""
import threading

import numpy as np
import pytest

from conftest import T16
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", ["batched", "mixed"])
def test_threads_share_a_context(native, gpu_ctx, form):
    import torch
    ctx = gpu_ctx(T16)
    nthreads, n, reps = 4, 1 << 16, 6
    inputs = [native.state_to_torch(W.mixed_batch(n, n_couples=16, seed=300 + k, id0=k * n)) for k in range(nthreads)]
    unif = [native.fill_uniforms(s["id"], 32, 5) for s in inputs]
    # one after another, on the default stream
    ref = []
    for k in range(nthreads):
        out, res = native.empty_state_torch(n), native.alloc_out_torch(n)
        ctx.step(inputs[k], out, unif[k], 32, 5, res, form=form)
        torch.cuda.synchronize()
        ref.append((native.to_numpy(out), native.to_numpy(res)))
    # at once: each thread steps its batch `reps` times on its own stream
    got = [None] * nthreads
    errors = []

    def work(k):
        try:
            torch.cuda.set_device(0)
            stream = torch.cuda.Stream()
            out, res = native.empty_state_torch(n), native.alloc_out_torch(n)
            torch.cuda.synchronize()
            for _ in range(reps):
                ctx.step(inputs[k], out, unif[k], 32, 5, res, form=form, stream=stream)
            stream.synchronize()
            got[k] = (native.to_numpy(out), native.to_numpy(res))
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(nthreads)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for k in range(nthreads):
        for key in ref[k][0]:
            assert np.array_equal(ref[k][0][key], got[k][0][key], equal_nan=True), (k, key)
        for key in ref[k][1]:
            assert np.array_equal(ref[k][1][key], got[k][1][key], equal_nan=True), (k, key)
