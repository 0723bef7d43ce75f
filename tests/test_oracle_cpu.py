"""CPU tests: the oracle pinned to the reference.

* the CPU port reproduces every golden vector written by the reference itself
  (tests/golden/make_golden.py) bit for bit;
* where the reference sources are present, the port and the reference agree on
  larger fresh batches too;
* Philox4x32-10 known-answer vectors (Random123 kat_vectors) for every
  implementation of the stream contract.
"""
import numpy as np
import pytest

from conftest import T3, T16, golden_res, golden_state, load_golden
from g4hepem_gb300 import workload as W
from oracle import oracle as O
from parity import compare_steps, energy_balance

KAT = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
       ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
       ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]


def test_philox_known_answers_numpy():
    for ctr, key, want in KAT:
        got = W.philox4x32_10(*[np.array([c], dtype=np.uint32) for c in ctr], key[0], key[1])
        assert tuple(int(g[0]) for g in got) == want


def test_philox_streams_agree(port):
    p = port(T3)
    ids = np.array([0, 1, 7, 123456, 2**31 - 1], dtype=np.int32)
    a = W.philox_uniforms(0xDEADBEEF12345678, ids, 33)
    b = p.fill_uniforms(ids, 33, 0xDEADBEEF12345678).reshape(len(ids), 33)
    assert np.array_equal(a, b)
    assert a.min() > 0.0 and a.max() < 1.0


def test_port_vdt_matches_reference_golden(port):
    g = load_golden("vdt.npz")
    p = port(T3)
    assert np.array_equal(p.vdt_log(g["x_log"]), g["y_log"], equal_nan=True)
    assert np.array_equal(p.vdt_exp(g["x_exp"]), g["y_exp"], equal_nan=True)


def test_port_lookups_match_reference_golden(port):
    g = load_golden("lookup_3couples.npz")
    p = port(T3)
    for pos in (0, 1):
        got = p.electron_lookup(g["ekin"], g["imc"], bool(pos))
        for k, v in got.items():
            assert np.array_equal(v, g[f"p{pos}_{k}"]), (pos, k)


@pytest.mark.parametrize("prefix,table", [("s1_", T3), ("s2_", T3), ("w_", T3), ("r_", T16)])
def test_port_steps_match_reference_golden(port, prefix, table):
    name = "step_16couples.npz" if table == T16 else "step_3couples.npz"
    g = load_golden(name)
    seeds = {"s1_": 0, "s2_": 1, "w_": 2, "r_": 0}
    seed = int(g["seed"][0]) + seeds[prefix]
    nu = int(g["nu"][0])
    st = golden_state(g, prefix, "in")
    u = W.philox_uniforms(seed, st["id"], nu)
    out, res = port(table).step(st, u, nu, seed)
    ref_out = golden_state(g, prefix, "out")
    ref_res = golden_res(g, prefix)
    # the port is a restatement of the reference on the same host libm:
    # everything is bit-identical
    for k in ref_out:
        assert np.array_equal(out[k], ref_out[k]), k
    for k in ref_res:
        assert np.array_equal(res[k], ref_res[k]), k
    rep, ok = compare_steps(ref_out, ref_res, out, res)
    assert ok, rep


def test_port_step_limit_cross_sections_match_reference_golden(port):
    """The HowFarToDiscreteInteraction inputs: restricted ioni and brem cross
    sections for stepping, e+ annihilation, e-nuclear and the transport mean
    free path (the reference's TestXSectionData quantities)."""
    for name, table, ekin_key in (("lookup_3couples.npz", T3, "ekin"), ("selectors_16couples.npz", T16, "s_ekin")):
        g = load_golden(name)
        p = port(table)
        for pos in (0, 1):
            got = p.electron_xs_stepping(g[ekin_key], g["imc"], bool(pos))
            for k, v in got.items():
                assert np.array_equal(v, g[f"p{pos}_step_{k}"]), (name, pos, k)


@pytest.mark.parametrize("name,table", [("selectors_3couples.npz", T3), ("selectors_16couples.npz", T16)])
def test_port_selectors_match_reference_golden(port, name, table):
    """Target-element selection for Seltzer-Berger and relativistic brem (e-
    and e+) and for conversion, and the gamma total cross section with the
    interaction it selects for a given uniform (the reference's
    TestElemSelectorData, TestGammaElemSelectorData and TestGammaXSectionData
    quantities), bit for bit."""
    g = load_golden(name)
    p = port(table)
    if "u" in g:
        g_imc, s_imc, gu, su = g["imc"], g["imc"], g["u"], g["u"]
    else:
        g_imc, s_imc, gu, su = g["g_imc"], np.zeros(len(g["s_ekin"]), np.int32), g["g_u"], g["s_u"]
    gx = p.gamma_xs(g["g_ekin"], g_imc, gu)
    assert np.array_equal(gx["xs_tot"], g["g_xs_tot"])
    assert np.array_equal(gx["winner"], g["g_winner"])
    assert np.array_equal(gx["xs_pe"], g["g_xs_pe"])
    assert np.array_equal(p.conv_select_target(g["s_ekin"], s_imc, su), g["conv"])
    for pos in (0, 1):
        for sb in (0, 1):
            got = p.brem_select_target(g["s_ekin"], s_imc, su, bool(pos), bool(sb))
            assert np.array_equal(got, g[f"brem_p{pos}_sb{sb}"]), (pos, sb)
    # every branch is exercised: each interaction and several target elements
    assert set(np.unique(g["g_winner"])) >= {0, 1, 2}
    assert len(np.unique(g["conv"])) >= 2


def test_golden_steps_conserve_energy():
    g = load_golden("step_3couples.npz")
    for prefix in ("s1_", "w_"):
        st, out, res = golden_state(g, prefix, "in"), golden_state(g, prefix, "out"), golden_res(g, prefix)
        bal = energy_balance(st, out, res)
        assert np.all(np.abs(bal) <= 1e-9 * np.maximum(st["ekin"], 1.0)), np.abs(bal).max()


def test_port_multithreaded_equals_single(port):
    p = port(T3)
    st = W.mixed_batch(20000, seed=3)
    u = W.philox_uniforms(9, st["id"], 64)
    o1, r1 = p.step(st, u, 64, 9)
    o2, r2 = p.step_mt(st, u, 64, 9, threads=4)
    for k in o1:
        assert np.array_equal(o1[k], o2[k])
    for k in r1:
        assert np.array_equal(r1[k], r2[k])


def test_port_matches_reference_fresh_batches(port, ref):
    """Larger batches than the golden files, both tables, both hosts' libm identical here."""
    for table, nc, n in ((T3, 3, 100000), (T16, 16, 50000)):
        st = W.mixed_batch(n, n_couples=nc, seed=31, emin=1e-3, emax=1e8)
        u = W.philox_uniforms(77, st["id"], 48)
        a_out, a_res = ref(table).step(st, u, 48, 77)
        b_out, b_res = port(table).step(st, u, 48, 77)
        for k in a_out:
            assert np.array_equal(a_out[k], b_out[k]), (table, k)
        for k in a_res:
            assert np.array_equal(a_res[k], b_res[k]), (table, k)


def test_port_in_place_equals_out_of_place(port):
    p = port(T3)
    st = W.mixed_batch(5000, seed=4)
    u = W.philox_uniforms(5, st["id"], 64)
    o1, r1 = p.step(st, u, 64, 5)
    st2 = O.copy_state(st)
    o2, r2 = p.step(st2, u, 64, 5, in_place=True)
    for k in o1:
        assert np.array_equal(o1[k], o2[k])


GEO_CASES = [("geosteps_3couples.npz", T3, "g1_", 0), ("geosteps_3couples.npz", T3, "g2_", 1),
             ("geosteps_16couples.npz", T16, "g1_", 0)]


def geo_inputs(g, prefix):
    """Pre-step state, transport (step fraction, direction after transport,
    post-step boundary status) of a geometry fixture."""
    st = golden_state(g, prefix, "in")
    nd = tuple(np.ascontiguousarray(g[f"{prefix}ndir_{c}"]) for c in "xyz")
    return st, g[f"{prefix}gfrac"], nd, np.ascontiguousarray(g[f"{prefix}post_bnd"])


@pytest.mark.parametrize("name,table,prefix,k", GEO_CASES)
def test_port_geometry_steps_match_reference_golden(port, name, table, prefix, k):
    """HowFar, a transport that shortens the step (some below the MSC
    geometrical length and below 1e-6 mm, some to 0), turns charged tracks and
    ends steps on a boundary, then Perform: the port equals the reference bit
    for bit, including the geometrical -> true length conversion
    (G4HepEmElectronManager.icc:171-203, :653-691) and the gamma boundary exit
    (G4HepEmProcess.cc:167-171)."""
    g = load_golden(name)
    seed, nu = int(g["seed"][k]), int(g["nu"][0])
    st, gfrac, nd, post = geo_inputs(g, prefix)
    u = W.philox_uniforms(seed, st["id"], nu)
    out, res, proposed = port(table).step_geom(st, u, nu, seed, gfrac, nd, post)
    assert np.array_equal(proposed, g[f"{prefix}proposed"])
    ref_out, ref_res = golden_state(g, prefix, "out"), golden_res(g, prefix)
    for key in ref_out:
        assert np.array_equal(out[key], ref_out[key]), key
    for key in ref_res:
        assert np.array_equal(res[key], ref_res[key]), key


def test_geometry_fixtures_cover_the_branches():
    """The fixtures exercise what a geometry-free step never reaches: e+-
    steps whose true length was recomputed from a shorter geometrical one
    (pstep > gstep, gstep < proposed), steps shortened below 1e-6 mm and to
    0, e+- steps ending on a boundary (no discrete interaction), and gammas
    taking the boundary exit (nia0 updated, no interaction)."""
    g = load_golden("geosteps_3couples.npz")
    for prefix in ("g1_", "g2_"):
        st, gfrac, _, post = geo_inputs(g, prefix)
        res = golden_res(g, prefix)
        ch = st["type"] != 2
        shortened = gfrac < 1.0
        conv = ch & shortened & (res["pstep"] > res["gstep"])
        assert conv.sum() > 500, prefix
        assert np.sum(ch & shortened & (res["gstep"] > 0) & (res["gstep"] < 1e-6)) > 20, prefix
        assert np.sum(gfrac == 0.0) > 20
        assert np.sum(ch & (post == 1) & (res["winner"] >= 0)) > 100
        gb = (st["type"] == 2) & (post == 1)
        assert gb.sum() > 200 and np.all(res["n_sec"][gb] == 0)
