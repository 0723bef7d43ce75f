"""Launch configuration of the batched form and its autotuner.

The configuration (threads per block and CTAs per SM of each stage kernel,
energy bins of the sort) changes where and with which neighbours a track is
stepped, never what is computed for it: every configuration must give
bit-identical results.
"""
import numpy as np
import pytest

from conftest import T16
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu

NU = 64
SEED = 4242


def _batched(native, ctx, sin, u, n):
    import torch
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step(sin, sout, u, NU, SEED, res, counters=cnt, form="batched")
    torch.cuda.synchronize()
    return native.to_numpy(sout), native.to_numpy(res), cnt.cpu().numpy()


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_autotuned_and_random_configs_are_bit_identical(native, gpu_ctx):
    ctx = gpu_ctx(T16)
    n = 1 << 18
    st = W.mixed_batch(n, n_couples=16, seed=71)
    sin = native.state_to_torch(st)
    u = native.fill_uniforms(sin["id"], NU, SEED)
    ctx.set_launch_config(None)
    base = _batched(native, ctx, sin, u, n)
    tuned = ctx.autotune(sin, u, NU, SEED, apply=True)
    assert ctx.launch_config()["block"] == tuned["block"]
    assert all(b in (128, 256, 512) for b in tuned["block"])
    assert tuned["sort_energy_bins"] in (8, 16, 32)
    got = _batched(native, ctx, sin, u, n)
    for x, y in zip(base, got):
        if isinstance(x, dict):
            _same(x, y)
        else:
            assert np.array_equal(x, y)
    rng = np.random.default_rng(5)
    for _ in range(3):
        cfg = {"block": [int(b) for b in rng.choice([128, 256, 512], 11)],
               "ctas_per_sm": [int(c) for c in rng.integers(0, 5, 11)],
               "sort_energy_bins": int(rng.choice([8, 16, 32]))}
        ctx.set_launch_config(cfg)
        got = _batched(native, ctx, sin, u, n)
        _same(base[0], got[0])
        _same(base[1], got[1])
        assert np.array_equal(base[2], got[2])
    ctx.set_launch_config(None)


def test_bad_launch_config_is_rejected(native, gpu_ctx):
    ctx = gpu_ctx(T16)
    good = ctx.launch_config()
    for bad in ({**good, "block": [96] + good["block"][1:]},
                {**good, "ctas_per_sm": [-1] + good["ctas_per_sm"][1:]},
                {**good, "sort_energy_bins": 12}):
        with pytest.raises(native.HepEmError) as e:
            ctx.set_launch_config(bad)
        assert e.value.code == 1
    assert ctx.launch_config() == good


@pytest.mark.parametrize("form", ["batched", "mixed"])
def test_table_l2_window_does_not_change_results(native, gpu_ctx, form):
    """The L2 persisting window over the tables changes where the table lines
    live, never a value: steps with and without it are bit-identical."""
    import torch
    ctx = gpu_ctx(T16)
    n = 1 << 17
    st = W.mixed_batch(n, n_couples=16, seed=73)
    sin = native.state_to_torch(st)
    u = native.fill_uniforms(sin["id"], NU, SEED)

    def run():
        sout = native.empty_state_torch(n)
        res = native.alloc_out_torch(n)
        cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
        ctx.step(sin, sout, u, NU, SEED, res, counters=cnt, form=form)
        torch.cuda.synchronize()
        return native.to_numpy(sout), native.to_numpy(res), cnt.cpu().numpy()

    try:
        on = ctx.set_table_l2_window(True)
        assert on >= 0
        with_w = run()
        assert ctx.set_table_l2_window(False) == 0
        without = run()
    finally:
        ctx.set_table_l2_window(False)
    _same(with_w[0], without[0])
    _same(with_w[1], without[1])
    assert np.array_equal(with_w[2], without[2])
