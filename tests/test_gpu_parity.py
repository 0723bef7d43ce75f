"""GPU parity: the CUDA path, called through the C-ABI, against the reference
golden vectors and the CPU port.

Tolerances (see parity.py): discrete outcomes identical; continuous values
within 1e-12 relative; direction cosines within 1e-12 absolute.
"""
import numpy as np
import pytest

from conftest import T3, T16, golden_res, golden_state, load_golden
from g4hepem_gb300 import workload as W
from parity import compare_steps, energy_balance

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def gpu_step(native, ctx, st_np, seed, nu, uniforms_np=None, in_place=False, form="plain"):
    torch = _torch()
    n = len(st_np["ekin"])
    sin = native.state_to_torch(st_np)
    sout = sin if in_place else native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    if uniforms_np is None:
        u = native.fill_uniforms(sin["id"], nu, seed)
    else:
        u = torch.from_numpy(np.ascontiguousarray(uniforms_np).reshape(-1)).cuda()
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step(sin, sout, u, nu, seed, res, counters=cnt, form=form)
    torch.cuda.synchronize()
    out = native.to_numpy(sout)
    if not in_place:
        for f in ("type", "imc", "id", "safety", "on_boundary"):
            out[f] = st_np[f]
    return out, native.to_numpy(res), cnt.cpu().numpy()


def test_vdt_log_exp_bit_exact_on_device(native, gpu_ctx):
    """log/exp through the lookup kernel's code path are covered below; here
    the range-lookup of a table at E gives VDTLog(E) implicitly."""
    g = load_golden("lookup_3couples.npz")
    ctx = gpu_ctx(T3)
    torch = _torch()
    ekin = torch.from_numpy(g["ekin"]).cuda()
    imc = torch.from_numpy(g["imc"]).cuda()
    for pos in (0, 1):
        out = ctx.electron_lookup(ekin, imc, positron=bool(pos))
        torch.cuda.synchronize()
        for k, v in out.items():
            got = v.cpu().numpy()
            assert np.array_equal(got, g[f"p{pos}_{k}"]), (pos, k, np.sum(got != g[f"p{pos}_{k}"]))


def test_lookup_16_couples_golden(native, gpu_ctx):
    g = load_golden("step_16couples.npz")
    ctx = gpu_ctx(T16)
    torch = _torch()
    out = ctx.electron_lookup(torch.from_numpy(g["l_ekin"]).cuda(), torch.from_numpy(g["l_imc"]).cuda())
    torch.cuda.synchronize()
    for k in ("xs_ioni", "xs_brem", "dedx", "range", "invrange_half"):
        assert np.array_equal(out[k].cpu().numpy(), g[f"l_{k}"]), k


def test_lookup_bad_inputs_give_nan_not_faults(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    torch = _torch()
    ekin = torch.tensor([1.0, -1.0, 0.0, float("nan"), 10.0], dtype=torch.float64, device="cuda")
    imc = torch.tensor([0, 0, 1, 2, 99], dtype=torch.int32, device="cuda")
    out = ctx.electron_lookup(ekin, imc)
    torch.cuda.synchronize()
    r = out["range"].cpu().numpy()
    assert np.isfinite(r[0]) and np.all(np.isnan(r[1:]))


@pytest.mark.parametrize("prefix,table", [("s1_", T3), ("s2_", T3), ("w_", T3), ("r_", T16)])
def test_step_matches_reference_golden(native, gpu_ctx, prefix, table):
    name = "step_16couples.npz" if table == T16 else "step_3couples.npz"
    g = load_golden(name)
    seed = int(g["seed"][0]) + {"s1_": 0, "s2_": 1, "w_": 2, "r_": 0}[prefix]
    nu = int(g["nu"][0])
    st = golden_state(g, prefix, "in")
    out, res, _ = gpu_step(native, gpu_ctx(table), st, seed, nu)
    rep, ok = compare_steps(golden_state(g, prefix, "out"), golden_res(g, prefix), out, res)
    print(prefix, rep)
    assert ok, rep


@pytest.mark.parametrize("table,nc", [(T3, 3), (T16, 16)])
def test_step_matches_port_200k(native, gpu_ctx, port, table, nc):
    st = W.mixed_batch(200000, n_couples=nc, seed=123)
    p = port(table)
    u = p.fill_uniforms(st["id"], 64, 4242)
    ref_out, ref_res = p.step_mt(st, u, 64, 4242, threads=8)
    out, res, cnt = gpu_step(native, gpu_ctx(table), st, 4242, 64)
    rep, ok = compare_steps(ref_out, ref_res, out, res)
    print(rep)
    assert ok, rep
    # counters agree with the per-track outputs
    assert cnt[0] == len(st["ekin"])
    assert cnt[1] == int(out["rng_cursor"].sum())
    assert cnt[3] == int(res["n_sec"].astype(np.int64).sum())


@pytest.mark.parametrize("form", ["plain", "batched", "mixed"])
def test_ragged_and_empty_batches(native, gpu_ctx, port, form):
    """Batch sizes that fill no warp, block or sort tile evenly (1 to 2,049
    tracks), and the empty batch, through every device form: the FP64 forms
    bit-exact with the port, the precision form with the port's discrete
    outcomes and energies within 1e-5."""
    ctx = gpu_ctx(T3)
    p = port(T3)
    for n in (1, 3, 31, 33, 257, 2049):
        st = W.mixed_batch(n, seed=100 + n)
        u = p.fill_uniforms(st["id"], 64, 77)
        ref_out, ref_res = p.step(st, u, 64, 77)
        out, res, cnt = gpu_step(native, ctx, st, 77, 64, form=form)
        if form == "mixed":
            for f in ("rng_cursor", "gauss_valid", "msc_first_step"):
                assert np.array_equal(ref_out[f], out[f]), (n, f)
            for f in ("winner", "n_sec", "flags"):
                assert np.array_equal(ref_res[f], res[f]), (n, f)
            a, b = ref_out["ekin"], out["ekin"]
            r = np.abs(a - b) / np.maximum(np.abs(a), 1e-300)
            assert np.all((a == b) | (r <= 1e-5)), (n, float(r.max()))
        else:
            rep, ok = compare_steps(ref_out, ref_res, out, res)
            assert ok, (n, rep)
        assert int(cnt[0]) == n
    st = W.mixed_batch(0, seed=1)
    out, res, cnt = gpu_step(native, ctx, st, 77, 64, form=form)
    assert len(out["ekin"]) == 0 and len(res["winner"]) == 0 and int(cnt[0]) == 0


def test_step_wide_energy_range_matches_port(native, gpu_ctx, port):
    """1 keV - 100 TeV: LPM brem/pair, RB brem, tracking cuts, at-rest annihilation."""
    st = W.mixed_batch(100000, seed=5, emin=1e-3, emax=1e8, frac=(0.4, 0.3, 0.3))
    rng = np.random.default_rng(8)
    st["on_boundary"] = (rng.random(len(st["ekin"])) < 0.2).astype(np.uint8)
    p = port(T3)
    u = p.fill_uniforms(st["id"], 24, 11)
    ref_out, ref_res = p.step_mt(st, u, 24, 11, threads=8)
    out, res, _ = gpu_step(native, gpu_ctx(T3), st, 11, 24)
    rep, ok = compare_steps(ref_out, ref_res, out, res)
    print(rep)
    assert ok, rep
    assert np.any(res["flags"] & 1), "expected some tracks to read past 24 buffered uniforms"


def test_in_place_equals_out_of_place(native, gpu_ctx):
    st = W.mixed_batch(50000, seed=6)
    a = gpu_step(native, gpu_ctx(T3), st, 3, 64)
    b = gpu_step(native, gpu_ctx(T3), st, 3, 64, in_place=True)
    for k in a[0]:
        assert np.array_equal(a[0][k], b[0][k], equal_nan=True), k
    for k in a[1]:
        assert np.array_equal(a[1][k], b[1][k], equal_nan=True), k


def test_host_entry_point_equals_device_entry_point(native, gpu_ctx):
    # 600,001 tracks: every chunk of the host pipeline in use, the last one ragged
    st = W.mixed_batch(600001, seed=9)
    out_d, res_d, _ = gpu_step(native, gpu_ctx(T3), st, 21, 64)
    u = W.philox_uniforms(21, st["id"], 64).reshape(-1)
    out_h = {k: np.empty_like(v) for k, v in st.items()}
    res_h = native.alloc_out_numpy(len(st["ekin"]))
    cnt = gpu_ctx(T3).step_host(st, out_h, u, 64, 21, res_h)
    for k in native.STATE_OUT_FIELDS:
        assert np.array_equal(out_d[k], out_h[k], equal_nan=True), k
    ns = res_d["n_sec"].astype(int)
    valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
    for k in res_d:
        a, b = (res_d[k][valid], res_h[k][valid]) if k.startswith("sec_") else (res_d[k], res_h[k])
        assert np.array_equal(a, b, equal_nan=True), k
    assert cnt.steps == len(st["ekin"])


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("in_place", [False, True])
def test_host_entry_point_pinned_buffers(native, gpu_ctx, mixed, in_place):
    """Pinned host buffers give the same results as pageable ones, in and out
    of place, with and without a uniform buffer, over several chunks (a
    ragged last one)."""
    import torch
    n = 300001
    st = W.mixed_batch(n, seed=29)
    ctx = gpu_ctx(T3)
    for nu in (0, 64):
        # pageable
        out_a = {k: np.empty_like(v) for k, v in st.items()}
        res_a = native.alloc_out_numpy(n)
        u = W.philox_uniforms(31, st["id"], nu).reshape(-1) if nu else None
        ctx.step_host(st, out_a, u, nu, 31, res_a, mixed=mixed)
        # pinned: torch tensors keep the pinned storage alive
        keep = []

        def pin(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            keep.append(t)
            return t.numpy()
        st_p = {k: pin(v) for k, v in st.items()}
        out_p = st_p if in_place else {k: pin(np.empty_like(v)) for k, v in st.items()}
        res_p = {k: pin(v) for k, v in native.alloc_out_numpy(n).items()}
        u_p = pin(u) if nu else None
        ctx.step_host(st_p, out_p, u_p, nu, 31, res_p, mixed=mixed)
        for k in native.STATE_OUT_FIELDS:
            assert np.array_equal(out_a[k], out_p[k], equal_nan=True), (nu, k)
        ns = res_a["n_sec"].astype(int)
        valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
        for k in res_a:
            a, b = (res_a[k][valid], res_p[k][valid]) if k.startswith("sec_") else (res_a[k], res_p[k])
            assert np.array_equal(a, b, equal_nan=True), (nu, k)


@pytest.mark.parametrize("mixed", [False, True])
def test_host_entry_point_without_buffer_draws_the_same_stream(native, gpu_ctx, mixed):
    # n_uniform = 0: every uniform comes from the on-device counter-based
    # stream, whose values the buffer holds in the device entry point: the
    # results are the same bit for bit
    import torch
    st = W.mixed_batch(30000, seed=19)
    ctx = gpu_ctx(T3)
    n = len(st["ekin"])
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], 64, 23)
    ctx.step(sin, sout, u, 64, 23, res, form="mixed" if mixed else "batched")
    torch.cuda.synchronize()
    out_d, res_d = native.to_numpy(sout), native.to_numpy(res)
    out_h = {k: np.empty_like(v) for k, v in st.items()}
    res_h = native.alloc_out_numpy(n)
    ctx.step_host(st, out_h, None, 0, 23, res_h, mixed=mixed)
    for k in native.STATE_OUT_FIELDS:
        assert np.array_equal(out_d[k], out_h[k], equal_nan=True), k
    # bit 0 of flags records draws past the buffer: every draw, without one
    assert np.array_equal(res_h["flags"] & 1, (out_d["rng_cursor"] > st["rng_cursor"]).astype(np.uint8))
    res_h["flags"] &= 0xFE
    res_d["flags"] &= 0xFE
    ns = res_d["n_sec"].astype(int)
    valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
    for k in res_d:
        a, b = (res_d[k][valid], res_h[k][valid]) if k.startswith("sec_") else (res_d[k], res_h[k])
        assert np.array_equal(a, b, equal_nan=True), k


def test_device_uniform_fill_matches_contract(native):
    torch = _torch()
    ids = torch.arange(0, 1000, dtype=torch.int32, device="cuda") * 7919
    u = native.fill_uniforms(ids, 37, 0xABCDEF).cpu().numpy().reshape(1000, 37)
    want = W.philox_uniforms(0xABCDEF, ids.cpu().numpy(), 37)
    assert np.array_equal(u, want)


def test_bad_track_inputs_are_flagged_not_faulted(native, gpu_ctx):
    st = W.mixed_batch(64, seed=1)
    st["imc"][3] = 99
    st["imc"][4] = -1
    st["ekin"][5] = -2.0
    st["ekin"][6] = np.nan
    st["type"][7] = 5
    out, res, _ = gpu_step(native, gpu_ctx(T3), st, 1, 64)
    for i in (3, 4, 5, 6, 7):
        assert res["flags"][i] & 4
    ok = np.ones(64, bool)
    ok[[3, 4, 5, 6, 7]] = False
    assert not np.any(res["flags"][ok] & 4)


# ---- full-size properties (the 4M mixed-track step) -----------------------------------
@pytest.fixture(scope="module")
def full_batch(native, gpu_ctx):
    n = 1 << 22
    st = W.mixed_batch(n, seed=2026)
    out, res, cnt = gpu_step(native, gpu_ctx(T3), st, 777, 64)
    return st, out, res, cnt


def test_full_size_energy_conservation(full_batch):
    st, out, res, _ = full_batch
    bal = energy_balance(st, out, res)
    assert np.all(np.abs(bal) <= 1e-9 * np.maximum(st["ekin"], 1.0)), float(np.abs(bal).max())


def test_full_size_unit_directions_and_sane_outputs(full_batch):
    st, out, res, _ = full_batch
    alive = out["ekin"] > 0
    nrm = np.sqrt(out["dir_x"] ** 2 + out["dir_y"] ** 2 + out["dir_z"] ** 2)
    assert np.all(np.abs(nrm[alive] - 1.0) < 1e-12)
    n = len(st["ekin"])
    ns = res["n_sec"].astype(int)
    valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
    snrm = np.sqrt(res["sec_dir_x"] ** 2 + res["sec_dir_y"] ** 2 + res["sec_dir_z"] ** 2)[valid]
    assert np.all(np.abs(snrm - 1.0) < 1e-12)
    assert np.all(res["sec_ekin"][valid] >= 0)
    assert np.all(res["gstep"] <= res["pstep"] + 1e-12 * np.abs(res["pstep"]))
    assert not np.any(res["flags"] & (2 | 4 | 8))
    assert n == len(ns)


def test_full_size_deterministic_and_order_independent(native, gpu_ctx, full_batch):
    st, out, res, _ = full_batch
    perm = np.random.default_rng(0).permutation(len(st["ekin"]))[: 1 << 20]
    sub = {k: np.ascontiguousarray(v[perm]) for k, v in st.items()}
    o2, r2, _ = gpu_step(native, gpu_ctx(T3), sub, 777, 64)
    for k in ("ekin", "dir_x", "nia0", "rng_cursor", "gauss_value"):
        assert np.array_equal(o2[k], out[k][perm], equal_nan=True), k
    for k in ("edep", "gstep", "pstep", "winner", "n_sec"):
        assert np.array_equal(r2[k], res[k][perm]), k


def test_full_size_sample_matches_port(port, full_batch):
    st, out, res, _ = full_batch
    idx = np.random.default_rng(1).choice(len(st["ekin"]), 65536, replace=False)
    sub = {k: np.ascontiguousarray(v[idx]) for k, v in st.items()}
    p = port(T3)
    u = p.fill_uniforms(sub["id"], 64, 777)
    ref_out, ref_res = p.step_mt(sub, u, 64, 777, threads=8)
    got_out = {k: v[idx] for k, v in out.items()}
    got_res = {k: (v.reshape(-1, 2)[idx].reshape(-1) if len(v) == 2 * len(st["ekin"]) else v[idx])
               for k, v in res.items()}
    rep, ok = compare_steps(ref_out, ref_res, got_out, got_res)
    assert ok, rep


# ---- batched form: same results as the plain form, bit for bit ------------------------------
@pytest.mark.parametrize("prefix,table", [("s1_", T3), ("s2_", T3), ("w_", T3), ("r_", T16)])
def test_batched_matches_reference_golden(native, gpu_ctx, prefix, table):
    name = "step_16couples.npz" if table == T16 else "step_3couples.npz"
    g = load_golden(name)
    seed = int(g["seed"][0]) + {"s1_": 0, "s2_": 1, "w_": 2, "r_": 0}[prefix]
    nu = int(g["nu"][0])
    st = golden_state(g, prefix, "in")
    out, res, _ = gpu_step(native, gpu_ctx(table), st, seed, nu, form="batched")
    rep, ok = compare_steps(golden_state(g, prefix, "out"), golden_res(g, prefix), out, res)
    assert ok, rep


@pytest.mark.parametrize("table,nc,emin,emax", [(T3, 3, 1.0, 1e4), (T3, 3, 1e-3, 1e8), (T16, 16, 1e-3, 1e5)])
def test_batched_equals_plain_bitwise(native, gpu_ctx, table, nc, emin, emax):
    st = W.mixed_batch(300000, n_couples=nc, seed=41, emin=emin, emax=emax)
    rng = np.random.default_rng(2)
    st["on_boundary"] = (rng.random(len(st["ekin"])) < 0.05).astype(np.uint8)
    st["imc"][:7] = [0, 1, -1, 99, 0, 0, 0]
    st["ekin"][4] = -1.0
    a_out, a_res, a_cnt = gpu_step(native, gpu_ctx(table), st, 99, 40)
    b_out, b_res, b_cnt = gpu_step(native, gpu_ctx(table), st, 99, 40, form="batched")
    for k in a_out:
        assert np.array_equal(a_out[k], b_out[k], equal_nan=True), k
    for k in a_res:
        if k.startswith("sec_"):
            ns = a_res["n_sec"].astype(int)
            valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
            assert np.array_equal(a_res[k][valid], b_res[k][valid]), k
        else:
            assert np.array_equal(a_res[k], b_res[k], equal_nan=True), k
    assert np.array_equal(a_cnt, b_cnt), (a_cnt, b_cnt)


@pytest.mark.parametrize("form", ["batched", "mixed"])
def test_batched_step_replays_from_a_cuda_graph(native, gpu_ctx, form):
    """The batched entry points (FP64 and precision form) are stream-capturable
    (their workspace is a stream-ordered allocation): capture once, replay,
    same results."""
    torch = _torch()
    st = W.mixed_batch(100000, seed=71)
    n = len(st["ekin"])
    ctx = gpu_ctx(T3)
    sin = native.state_to_torch(st)
    u = native.fill_uniforms(sin["id"], 64, 9)
    ref_out, ref_res = native.empty_state_torch(n), native.alloc_out_torch(n)
    ctx.step(sin, ref_out, u, 64, 9, ref_res, form=form)
    g_out, g_res = native.empty_state_torch(n), native.alloc_out_torch(n)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        ctx.step(sin, g_out, u, 64, 9, g_res, form=form)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        ctx.step(sin, g_out, u, 64, 9, g_res, form=form)
    for v in list(g_out.values()) + list(g_res.values()):
        v.zero_()
    graph.replay()
    graph.replay()
    torch.cuda.synchronize()
    a, b = native.to_numpy(ref_out), native.to_numpy(g_out)
    for k in native.STATE_OUT_FIELDS:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    ra, rb = native.to_numpy(ref_res), native.to_numpy(g_res)
    for k in ("edep", "gstep", "pstep", "winner", "n_sec", "flags"):
        assert np.array_equal(ra[k], rb[k]), k


def test_batched_in_place(native, gpu_ctx):
    st = W.mixed_batch(50000, seed=61)
    a = gpu_step(native, gpu_ctx(T3), st, 5, 64, form="batched")
    b = gpu_step(native, gpu_ctx(T3), st, 5, 64, in_place=True, form="batched")
    for k in a[0]:
        assert np.array_equal(a[0][k], b[0][k], equal_nan=True), k
    for k in ("edep", "winner", "n_sec", "flags"):
        assert np.array_equal(a[1][k], b[1][k]), k


def test_context_from_arena_image_is_identical(native, gpu_ctx):
    # the binary arena image loads to the same tables: same step, bit for bit
    ctx_json = gpu_ctx(T16)
    img = native.image_from_json(open(T16, "rb").read())
    ctx_img = native.Context(image=img)
    try:
        assert ctx_img.info() == ctx_json.info()
        st = W.mixed_batch(1 << 16, n_couples=16, seed=77)
        a = gpu_step(native, ctx_json, st, 5, 16, form="batched")
        b = gpu_step(native, ctx_img, st, 5, 16, form="batched")
        for x, y in zip(a[:2], b[:2]):
            for k in x:
                assert np.array_equal(x[k], y[k], equal_nan=True), k
        assert np.array_equal(a[2], b[2])
    finally:
        ctx_img.close()
