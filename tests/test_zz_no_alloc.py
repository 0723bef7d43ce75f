"""The allocation-free batched step, hepem_step_batched_noalloc.

It serves callers that cannot let a library allocate device memory (their
memory is owned by their own pool allocator, or their latency path must not
enter an allocator).  It must give the same results as hepem_step_batched, the
entry point that allocates its workspace, call after call: the shared static
workspace keeps the previous call's contents and must not leak into the next.
Named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import T3, T16
from g4hepem_gb300 import workload as W
from parity import compare_steps

pytestmark = pytest.mark.gpu


def _run(native, ctx, st_np, seed, nu, form):
    import torch
    n = len(st_np["ekin"])
    sin = native.state_to_torch(st_np)
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], nu, seed)
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step(sin, sout, u, nu, seed, res, counters=cnt, form=form)
    torch.cuda.synchronize()
    out = native.to_numpy(sout)
    for f in ("type", "imc", "id", "safety", "on_boundary"):
        out[f] = st_np[f]
    return out, native.to_numpy(res), cnt.cpu().numpy()


@pytest.mark.parametrize("order", ["three_then_sixteen", "sixteen_then_three"])
def test_noalloc_equals_allocating_entry_point_two_calls_in_a_row(native, gpu_ctx, order):
    # two calls in a row on different tables: the second call must not see
    # anything the first one left in the shared workspace.  The sixteen-couple
    # table has more sort keys than the three-couple one, so running it first
    # leaves a longer histogram behind than the next call uses.
    cases = [(T3, 3, 400000, 1.0, 1e4, 31), (T16, 16, 150000, 1e-3, 1e5, 32)]
    if order == "sixteen_then_three":
        cases = cases[::-1]
    for table, nc, n, emin, emax, seed in cases:
        st = W.mixed_batch(n, n_couples=nc, seed=seed, emin=emin, emax=emax)
        ref_out, ref_res, ref_cnt = _run(native, gpu_ctx(table), st, seed, 48, "batched")
        got_out, got_res, got_cnt = _run(native, gpu_ctx(table), st, seed, 48, "noalloc")
        rep, ok = compare_steps(ref_out, ref_res, got_out, got_res)
        assert ok, rep
        for k in ("ekin", "dir_x", "dir_y", "dir_z", "nia0", "rng_cursor", "gauss_value"):
            assert np.array_equal(ref_out[k], got_out[k]), k
        assert np.array_equal(ref_cnt, got_cnt)


def test_noalloc_rejects_batches_above_its_limit(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    n = native.NOALLOC_MAX_TRACKS + 1
    st = W.mixed_batch(n, seed=3)
    with pytest.raises(native.HepEmError) as e:
        _run(native, ctx, st, 1, 8, "noalloc")
    assert e.value.code == 1
    assert "exceeds the maximum" in str(e.value)
    # the context stays usable after the rejection
    small = W.mixed_batch(1000, seed=4)
    a = _run(native, ctx, small, 2, 16, "noalloc")
    b = _run(native, ctx, small, 2, 16, "batched")
    assert np.array_equal(a[0]["ekin"], b[0]["ekin"])


class _DefaultPool:
    """The device's default memory pool (the one cudaMallocAsync draws from),
    read through the CUDA runtime: its bytes in use and their high-water mark."""

    def __init__(self, dev=0):
        for name in ("libcudart.so.13", "libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = C.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def used(self):
        return self._get(7)  # cudaMemPoolAttrUsedMemCurrent

    def used_high(self):
        return self._get(8)  # cudaMemPoolAttrUsedMemHigh

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, 8, C.byref(zero)) == 0


def test_noalloc_allocates_no_device_memory(native, gpu_ctx):
    """The entry point's defining property: its calls take no memory from the
    device's default pool, while hepem_step_batched's stream-ordered workspace
    does (which shows that the measurement sees such allocations)."""
    import torch
    ctx = gpu_ctx(T3)
    n = 200000
    st = W.mixed_batch(n, seed=8)
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], 48, 8)
    torch.cuda.synchronize()
    pool = _DefaultPool(torch.cuda.current_device())
    base = pool.used()
    pool.reset_high()
    ctx.step(sin, sout, u, 48, 8, res, form="batched")
    torch.cuda.synchronize()
    assert pool.used_high() > base
    assert pool.used() == base
    pool.reset_high()
    for _ in range(3):
        ctx.step(sin, sout, u, 48, 8, res, form="noalloc")
    torch.cuda.synchronize()
    assert pool.used_high() == base and pool.used() == base
