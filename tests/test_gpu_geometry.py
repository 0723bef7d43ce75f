"""HowFar and Perform as two calls with a caller's transport between them
(hepem_howfar / hepem_perform), through the C-ABI, on the GPU.

The reference client calls HowFar, lets the geometry move the track, then
Perform (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-197).  The golden
fixtures geosteps_*.npz are the reference's own results for steps that
transport shortened (below the MSC geometrical length, below 1e-6 mm, to 0),
turned (charged tracks) and ended on a boundary.  Checked here:
  * the FP64 forms (plain, batched): the proposed step bit-identical to the
    reference's, and the step against the golden results with the tolerances
    of parity.py (discrete identical, continuous within 1e-12);
  * the precision form against the FP64 plain form on the same transport
    (discrete identical, continuous within 1e-5, as tests/test_gpu_mixed.py);
  * unchanged transport: HowFar + Perform equals the fused hepem_step* of the
    same form bit for bit, counters included;
  * in-place Perform, and the host-buffer calls, equal the device calls.
"""
import numpy as np
import pytest

from conftest import T3, T16, golden_res, golden_state, load_golden
from g4hepem_gb300 import workload as W
from parity import compare_steps

pytestmark = pytest.mark.gpu

GEO_CASES = [("geosteps_3couples.npz", T3, "g1_", 0), ("geosteps_3couples.npz", T3, "g2_", 1),
             ("geosteps_16couples.npz", T16, "g1_", 0)]


def _torch():
    import torch
    return torch


def geo_inputs(g, prefix):
    st = golden_state(g, prefix, "in")
    nd = tuple(np.ascontiguousarray(g[f"{prefix}ndir_{c}"]) for c in "xyz")
    return st, g[f"{prefix}gfrac"], nd, np.ascontiguousarray(g[f"{prefix}post_bnd"])


def split_step(native, ctx, st, seed, nu, gfrac, nd, post, form, in_place=False, shortened=None):
    """howfar -> transport (step gfrac * proposed, or shortened[i] where
    gfrac[i] < 1 if given; direction nd; post-step boundary status) ->
    perform; returns (proposed, out state, res, counters of howfar, counters
    of perform) as numpy."""
    torch = _torch()
    n = len(st["ekin"])
    sin = native.state_to_torch(st)
    u = native.fill_uniforms(sin["id"], nu, seed)
    c1 = torch.zeros(13, dtype=torch.int64, device="cuda")
    c2 = torch.zeros(13, dtype=torch.int64, device="cuda")
    gstep, limits = ctx.howfar(sin, u, nu, seed, counters=c1, form=form)
    proposed = gstep.clone()
    gstep *= torch.from_numpy(np.ascontiguousarray(gfrac)).cuda()
    if shortened is not None:
        made = np.where(gfrac < 1.0, shortened, gstep.cpu().numpy())
        gstep.copy_(torch.from_numpy(made))
    for c, a in zip("xyz", nd):
        sin[f"dir_{c}"].copy_(torch.from_numpy(a))
    sin["on_boundary"].copy_(torch.from_numpy(post))
    sout = sin if in_place else native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    ctx.perform(sin, sout, gstep, limits, u, nu, seed, res, counters=c2, form=form)
    torch.cuda.synchronize()
    out = native.to_numpy(sout)
    if not in_place:
        for f in ("type", "imc", "id", "safety", "on_boundary"):
            out[f] = native.to_numpy({f: sin[f]})[f]
    return proposed.cpu().numpy(), out, native.to_numpy(res), c1.cpu().numpy(), c2.cpu().numpy()


@pytest.mark.parametrize("form", ["plain", "batched"])
@pytest.mark.parametrize("name,table,prefix,k", GEO_CASES)
def test_geometry_steps_match_reference_golden(native, gpu_ctx, name, table, prefix, k, form):
    g = load_golden(name)
    seed, nu = int(g["seed"][k]), int(g["nu"][0])
    st, gfrac, nd, post = geo_inputs(g, prefix)
    proposed, out, res, _, _ = split_step(native, gpu_ctx(table), st, seed, nu, gfrac, nd, post, form)
    assert np.array_equal(proposed, g[f"{prefix}proposed"]), np.sum(proposed != g[f"{prefix}proposed"])
    ref_out, ref_res = golden_state(g, prefix, "out"), golden_res(g, prefix)
    rep, ok = compare_steps(ref_out, ref_res, out, res)
    assert ok, rep
    # energies, steps and deposits bit for bit (only sin/cos differ in the last bits)
    for key in ("ekin", "nia0", "nia1", "msc_init_range", "rng_cursor", "on_boundary"):
        assert np.array_equal(out[key], ref_out[key]), key
    for key in ("edep", "gstep", "pstep", "winner", "n_sec"):
        assert np.array_equal(res[key], ref_res[key]), key


@pytest.mark.parametrize("name,table,prefix,k", GEO_CASES)
def test_geometry_steps_precision_form(native, gpu_ctx, name, table, prefix, k):
    """The precision form's split step against the FP64 plain split step on the
    same transport (step fraction, direction, boundary status)."""
    from test_gpu_mixed import compare
    g = load_golden(name)
    seed, nu = int(g["seed"][k]), int(g["nu"][0])
    st, gfrac, nd, post = geo_inputs(g, prefix)
    ctx = gpu_ctx(table)
    p64, o64, r64, _, c64 = split_step(native, ctx, st, seed, nu, gfrac, nd, post, "plain")
    # the geometry makes the same shortened steps whatever the physics form
    p32, o32, r32, _, c32 = split_step(native, ctx, st, seed, nu, gfrac, nd, post, "mixed",
                                       shortened=gfrac * p64)
    assert np.max(np.abs(p32 - p64) / np.maximum(np.abs(p64), 1e-300)) <= 1e-5
    st_after = dict(st)
    st_after["on_boundary"] = post
    c64 = np.concatenate([c64[:12], [0]])
    compare(st_after, (o64, r64, c64), (o32, r32, np.concatenate([c32[:12], [0]])))


@pytest.mark.parametrize("form,fused", [("plain", "plain"), ("batched", "batched"), ("mixed", "mixed")])
@pytest.mark.parametrize("table,nc", [(T3, 3), (T16, 16)])
def test_unchanged_transport_equals_fused_step(native, gpu_ctx, form, fused, table, nc):
    """howfar + perform with the proposed step, the direction and the boundary
    status unchanged is hepem_step of the same form, bit for bit."""
    torch = _torch()
    ctx = gpu_ctx(table)
    n = 1 << 16
    st = W.mixed_batch(n, n_couples=nc, seed=44, emin=1e-3, emax=1e6)
    st["on_boundary"] = (np.random.default_rng(2).random(n) < 0.1).astype(np.uint8)
    nd = (st["dir_x"], st["dir_y"], st["dir_z"])
    _, out, res, c1, c2 = split_step(native, ctx, st, 5, 32, np.ones(n), nd, st["on_boundary"], form)
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    r2 = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], 32, 5)
    cf = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step(sin, sout, u, 32, 5, r2, counters=cf, form=fused)
    torch.cuda.synchronize()
    fo, fr, cf = native.to_numpy(sout), native.to_numpy(r2), cf.cpu().numpy()
    for key in out:
        assert np.array_equal(out[key], fo[key]), key
    for key in res:
        assert np.array_equal(res[key], fr[key]), key
    # counters: the step's uniforms are HowFar's plus Perform's
    assert c2[0] == cf[0] == n
    assert c1[1] + c2[1] == cf[1]
    assert np.array_equal(c2[3:12], cf[3:12])


@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_in_place_perform_and_host_buffers(native, gpu_ctx, form):
    g = load_golden("geosteps_3couples.npz")
    seed, nu = int(g["seed"][0]), int(g["nu"][0])
    st, gfrac, nd, post = geo_inputs(g, "g1_")
    ctx = gpu_ctx(T3)
    _, a_out, a_res, _, _ = split_step(native, ctx, st, seed, nu, gfrac, nd, post, form)
    _, b_out, b_res, _, _ = split_step(native, ctx, st, seed, nu, gfrac, nd, post, form, in_place=True)
    for key in a_out:
        assert np.array_equal(a_out[key], b_out[key]), key
    for key in a_res:
        assert np.array_equal(a_res[key], b_res[key]), key
    # host buffers
    n = len(st["ekin"])
    u = W.philox_uniforms(seed, st["id"], nu).reshape(-1)
    gstep, limits, _ = ctx.howfar_host(st, u, nu, seed, form=form)
    st2 = {k: v.copy() for k, v in st.items()}
    st2["dir_x"], st2["dir_y"], st2["dir_z"] = (a.copy() for a in nd)
    st2["on_boundary"] = post.copy()
    out = {k: np.empty_like(v) for k, v in st2.items()}
    res = native.alloc_out_numpy(n)
    ctx.perform_host(st2, out, gstep * gfrac, limits, u, nu, seed, res, form=form)
    for key in a_out:
        assert np.array_equal(a_out[key], out[key]), key
    for key in a_res:
        assert np.array_equal(a_res[key], res[key]), key


def test_split_rejects_bad_arguments(native, gpu_ctx):
    torch = _torch()
    ctx = gpu_ctx(T3)
    st = native.state_to_torch(W.mixed_batch(8, seed=1))
    u = native.fill_uniforms(st["id"], 4, 1)
    L = native.lib()
    sin = native.make_state_struct(st)
    g = torch.empty(8, dtype=torch.float64, device="cuda")
    lim = torch.empty(L.hepem_step_limit_bytes(8), dtype=torch.uint8, device="cuda")
    import ctypes as C
    assert L.hepem_howfar(ctx.h, 7, 8, C.byref(sin), native._ptr(u), 4, 1, native._ptr(g), native._ptr(lim), None,
                          native._stream_ptr(None)) == 1
    assert L.hepem_howfar(ctx.h, 0, 8, C.byref(sin), native._ptr(u), 4, 1, None, native._ptr(lim), None,
                          native._stream_ptr(None)) == 1
    assert L.hepem_howfar(ctx.h, 0, 0, C.byref(sin), None, 0, 1, None, None, None, native._stream_ptr(None)) == 0
