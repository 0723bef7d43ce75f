"""Single functions of the path on the GPU, called through the C-ABI as the
reference's own device tests call them, against the reference's golden
vectors (tests/golden/make_golden.py):

  hepem_electron_xs_stepping  testing/ElectronXSections (TestXSectionData)
  hepem_brem_select_target    testing/ElectronTargetElementSelector (SB and RB, e- and e+)
  hepem_conv_select_target    testing/GammaTargetElementSelector
  hepem_gamma_xs              testing/GammaXSections (total cross section and selected interaction)

FP64 (precision 0): bit-identical.  FP32 (precision 1, the code of the
precision form): selections identical, cross sections within 1e-5 relative.
"""
import numpy as np
import pytest

from conftest import T3, T16, load_golden

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _np(x):
    return x.cpu().numpy()


def rel(a, b):
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    r[a == b] = 0.0
    return r


def selector_inputs(g):
    if "u" in g:
        return g["imc"], g["imc"], g["u"], g["u"]
    return g["g_imc"], np.zeros(len(g["s_ekin"]), np.int32), g["g_u"], g["s_u"]


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name,table", [("selectors_3couples.npz", T3), ("selectors_16couples.npz", T16)])
def test_selectors_and_gamma_xs_golden(native, gpu_ctx, name, table, mixed):
    g = load_golden(name)
    ctx = gpu_ctx(table)
    g_imc, s_imc, gu, su = selector_inputs(g)
    gx = ctx.gamma_xs(_t(g["g_ekin"]), _t(g_imc.astype(np.int32)), _t(gu), mixed=mixed)
    win = _np(gx["winner"])
    assert np.array_equal(win, g["g_winner"]), np.sum(win != g["g_winner"])
    # the photoelectric cross section the photoelectric model uses is FP64 in
    # both forms; the precision form's translation unit contracts FP64
    # multiply-adds, so there it agrees to a few ulp
    pe = _np(gx["xs_pe"])
    if mixed:
        assert np.array_equal(pe == 0, g["g_xs_pe"] == 0) and rel(pe, g["g_xs_pe"]).max() <= 1e-15
    else:
        assert np.array_equal(pe, g["g_xs_pe"])
    tot = _np(gx["xs_tot"])
    if mixed:
        assert rel(tot, g["g_xs_tot"]).max() <= TOL32
    else:
        assert np.array_equal(tot, g["g_xs_tot"])
    es, si, us = _t(g["s_ekin"]), _t(s_imc.astype(np.int32)), _t(su)
    conv = _np(ctx.conv_select_target(es, si, us, mixed=mixed))
    assert np.array_equal(conv, g["conv"]), np.sum(conv != g["conv"])
    for pos in (0, 1):
        for sb in (0, 1):
            got = _np(ctx.brem_select_target(es, si, us, positron=bool(pos), sb=bool(sb), mixed=mixed))
            want = g[f"brem_p{pos}_sb{sb}"]
            assert np.array_equal(got, want), (pos, sb, np.sum(got != want))
    # several target elements and every interaction are exercised
    assert len(np.unique(g["conv"])) >= 2 and set(np.unique(g["g_winner"])) >= {0, 1, 2}


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name,table,ekin_key", [("lookup_3couples.npz", T3, "ekin"),
                                                 ("selectors_16couples.npz", T16, "s_ekin")])
def test_step_limit_cross_sections_golden(native, gpu_ctx, name, table, ekin_key, mixed):
    g = load_golden(name)
    ctx = gpu_ctx(table)
    e, imc = _t(g[ekin_key]), _t(g["imc"].astype(np.int32))
    worst = 0.0
    for pos in (0, 1):
        got = ctx.electron_xs_stepping(e, imc, positron=bool(pos), mixed=mixed)
        for k, v in got.items():
            want = g[f"p{pos}_step_{k}"]
            v = _np(v)
            if mixed:
                r = rel(v, want)
                worst = max(worst, float(r.max()))
                assert r.max() <= TOL32, (pos, k, float(r.max()))
                assert np.array_equal(v == 0, want == 0), (pos, k)
            else:
                assert np.array_equal(v, want), (pos, k, np.sum(v != want))
    if mixed:
        print(f"\nFP32 step-limit cross sections: max relative error {worst:.2e}")


def test_function_checks_reject_bad_inputs(native, gpu_ctx):
    ctx = gpu_ctx(T3)
    e = _t(np.array([1.0, -1.0, 10.0]))
    imc = _t(np.array([0, 0, 99], np.int32))
    u = _t(np.array([0.5, 0.5, 0.5]))
    xs = _np(ctx.electron_xs_stepping(e, imc)["xs_ioni"])
    assert np.isfinite(xs[0]) and np.all(np.isnan(xs[1:]))
    assert list(_np(ctx.conv_select_target(e, imc, u))[1:]) == [-1, -1]
    assert list(_np(ctx.gamma_xs(e, imc, u)["winner"])[1:]) == [-1, -1]
