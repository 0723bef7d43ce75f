"""Write the golden vectors of tests/golden/ by running the REFERENCE itself.

Usage (where the reference sources are present):
    python tests/golden/make_golden.py

It builds oracle/_ref/libhepem_ref.so from the reference sources (oracle/Makefile),
loads the committed synthetic tables through the reference's own
G4HepEmStateFromJson, and records inputs and outputs of the reference
functions: VDT log/exp, the electron table lookups, step-limit cross
sections, target-element selectors (brem SB/RB for e- and e+, conversion),
gamma cross sections and interaction selection, on three and on sixteen
couples, and full HowFar+Perform steps (fresh tracks, a second step that
carries MSC/Gauss/RNG state, boundary and safety variants, and a 16-couple
table with two regions), and steps whose geometry shortens the proposed
step, turns charged tracks and ends steps on a boundary between HowFar and
Perform (`--only-geometry` writes just those).  Uniform streams are not stored: they are the Philox
streams of the C-ABI contract and are regenerated from (seed, id).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402
from g4hepem_gb300 import workload as W  # noqa: E402
from g4hepem_gb300.tables import synth  # noqa: E402

DATA = os.path.join(REPO, "g4hepem_gb300", "data")
T3 = os.path.join(DATA, "three_couples_0.7mm.json")
T16 = os.path.join(DATA, "random16_two_regions.json")
SEED = 20261203
NU = 64


def save(name, **arrs):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrs)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


def step_fixture(ref, state, seed, nu=NU, prefix=""):
    u = W.philox_uniforms(seed, state["id"], nu)
    out, res = ref.step(state, u, nu, seed)
    d = {}
    for k, v in state.items():
        d[f"{prefix}in_{k}"] = v
    for k, v in out.items():
        d[f"{prefix}out_{k}"] = v
    for k, v in res.items():
        d[f"{prefix}res_{k}"] = v
    return d, out


def geom_fixture(ref, state, seed, tseed, nu=NU, prefix=""):
    """HowFar, a caller's transport (workload.transport), Perform."""
    u = W.philox_uniforms(seed, state["id"], nu)
    gfrac, nd, post = W.transport(state, tseed)
    out, res, proposed = ref.step_geom(state, u, nu, seed, gfrac, nd, post)
    d = {f"{prefix}gfrac": gfrac, f"{prefix}ndir_x": nd[0], f"{prefix}ndir_y": nd[1], f"{prefix}ndir_z": nd[2],
         f"{prefix}post_bnd": post, f"{prefix}proposed": proposed}
    for k, v in state.items():
        d[f"{prefix}in_{k}"] = v
    for k, v in out.items():
        d[f"{prefix}out_{k}"] = v
    for k, v in res.items():
        d[f"{prefix}res_{k}"] = v
    return d, out


def geometry_fixtures():
    """Geometry-limited steps: HowFar, transport that shortens the step,
    turns charged tracks and sets the post-step boundary status, Perform; a
    first and a second step on three couples, one step on sixteen."""
    ref = O.RefLib().load(T3)
    st = wide_batch(8192, 3, 31)
    d1, out1 = geom_fixture(ref, st, SEED + 10, 101, prefix="g1_")
    st2 = O.copy_state(out1)
    st2["rng_cursor"] = np.zeros_like(st2["rng_cursor"])
    alive = st2["ekin"] > 0
    st2 = {k: np.ascontiguousarray(v[alive]) for k, v in st2.items()}
    d2, _ = geom_fixture(ref, st2, SEED + 11, 102, prefix="g2_")
    save("geosteps_3couples.npz", seed=np.array([SEED + 10, SEED + 11]), nu=np.array([NU]), **d1, **d2)
    ref16 = O.RefLib().load(T16)
    st = wide_batch(8192, 16, 32)
    d3, _ = geom_fixture(ref16, st, SEED + 12, 103, prefix="g1_")
    save("geosteps_16couples.npz", seed=np.array([SEED + 12]), nu=np.array([NU]), **d3)


def wide_batch(n, n_couples, seed):
    """Energies log-uniform 1 keV - 100 TeV, 10% on a boundary, 10% zero safety."""
    st = W.mixed_batch(n, n_couples=n_couples, seed=seed, emin=1e-3, emax=1e8, frac=(0.4, 0.4, 0.2))
    rng = np.random.default_rng(seed + 1)
    st["on_boundary"] = (rng.random(n) < 0.1).astype(np.uint8)
    st["safety"] = np.where(rng.random(n) < 0.1, 0.0, st["safety"])
    return st


def main():
    if "--only-geometry" in sys.argv:
        if not O.build_ref():
            raise SystemExit("could not build oracle/_ref (reference sources missing?)")
        geometry_fixtures()
        return
    if not os.path.exists(T16):
        regions = [dict(), dict(fIsMSCMinimalStepLimit=True, fIsELossFluctuation=False, fLinELossLimit=0.02,
                                fFinalRange=0.1, fDRoverRange=0.8, fMSCRangeFactor=0.08)]
        synth.write(synth.random_couple_state(16, seed=1234, regions=regions), T16)
    if not O.build_ref():
        raise SystemExit("could not build oracle/_ref (reference sources missing?)")
    ref = O.RefLib().load(T3)

    # VDT log / exp
    r = np.random.default_rng(1)
    xl = np.concatenate([np.exp(r.uniform(-700, 700, 3000)), r.uniform(0, 1, 1000), [1.0, 2.0, 0.5, 1e-310]])
    xe = np.concatenate([r.uniform(-720, 720, 3000), r.uniform(-1, 1, 1000), [0.0, -0.0, 708.0, -708.0]])
    save("vdt.npz", x_log=xl, y_log=ref.vdt_log(xl), x_exp=xe, y_exp=ref.vdt_exp(xe))

    # electron table lookups + step-limit cross sections
    ekin, imc = W.electron_lookup_batch(8192, seed=11)
    d = dict(ekin=ekin, imc=imc)
    for pos in (0, 1):
        for k, v in ref.electron_lookup(ekin, imc, bool(pos)).items():
            d[f"p{pos}_{k}"] = v
        for k, v in ref.electron_xs_stepping(ekin, imc, bool(pos)).items():
            d[f"p{pos}_step_{k}"] = v
    save("lookup_3couples.npz", **d)

    # selectors and gamma interaction choice
    rr = np.random.default_rng(5)
    eg = np.exp(rr.uniform(np.log(1e-3), np.log(1e8), 8192))
    ig = rr.integers(0, 3, 8192).astype(np.int32)
    ug = rr.random(8192)
    gx = ref.gamma_xs(eg, ig, ug)
    es = np.exp(rr.uniform(np.log(0.1), np.log(1e8), 8192))
    us = rr.random(8192)
    d = dict(g_ekin=eg, g_imc=ig, g_u=ug, g_xs_tot=gx["xs_tot"], g_xs_pe=gx["xs_pe"], g_winner=gx["winner"],
             s_ekin=es, s_u=us, conv=ref.conv_select_target(es, np.zeros(8192, np.int32), us))
    for pos in (0, 1):
        for sb in (0, 1):
            d[f"brem_p{pos}_sb{sb}"] = ref.brem_select_target(es, np.zeros(8192, np.int32), us, bool(pos), bool(sb))
    save("selectors_3couples.npz", **d)

    # full steps, three couples: the 45/45/10 mix, a second step, a wide-range batch
    st = W.mixed_batch(8192, seed=7)
    d1, out1 = step_fixture(ref, st, SEED, prefix="s1_")
    # second step: continue the same tracks (alive ones keep their state)
    st2 = O.copy_state(out1)
    st2["rng_cursor"] = np.zeros_like(st2["rng_cursor"])
    alive = st2["ekin"] > 0
    st2 = {k: np.ascontiguousarray(v[alive]) for k, v in st2.items()}
    d2, _ = step_fixture(ref, st2, SEED + 1, prefix="s2_")
    d3, _ = step_fixture(ref, wide_batch(8192, 3, 99), SEED + 2, prefix="w_")
    save("step_3couples.npz", seed=np.array([SEED]), nu=np.array([NU]), **d1, **d2, **d3)

    # sixteen random couples, two regions (minimal MSC step limit, no fluctuation)
    ref16 = O.RefLib().load(T16)
    st = W.mixed_batch(8192, n_couples=16, seed=17, emin=1e-3, emax=1e5)
    rng = np.random.default_rng(3)
    st["on_boundary"] = (rng.random(8192) < 0.1).astype(np.uint8)
    d4, _ = step_fixture(ref16, st, SEED + 3, prefix="r_")
    ekin, imc = W.electron_lookup_batch(4096, n_couples=16, seed=12)
    lk = {f"l_{k}": v for k, v in ref16.electron_lookup(ekin, imc).items()}
    save("step_16couples.npz", seed=np.array([SEED + 3]), nu=np.array([NU]), l_ekin=ekin, l_imc=imc, **lk, **d4)

    # selectors, gamma cross sections and step-limit cross sections over the
    # sixteen couples (1-4 elements each, random couple per input)
    rr = np.random.default_rng(6)
    n16 = 16384
    eg = np.exp(rr.uniform(np.log(1e-3), np.log(1e8), n16))
    es = np.exp(rr.uniform(np.log(0.1), np.log(1e8), n16))
    ic = rr.integers(0, 16, n16).astype(np.int32)
    u = rr.random(n16)
    gx = ref16.gamma_xs(eg, ic, u)
    d = dict(g_ekin=eg, s_ekin=es, imc=ic, u=u, g_xs_tot=gx["xs_tot"], g_xs_pe=gx["xs_pe"],
             g_winner=gx["winner"], conv=ref16.conv_select_target(es, ic, u))
    for pos in (0, 1):
        for sb in (0, 1):
            d[f"brem_p{pos}_sb{sb}"] = ref16.brem_select_target(es, ic, u, bool(pos), bool(sb))
        for k, v in ref16.electron_xs_stepping(es, ic, bool(pos)).items():
            d[f"p{pos}_step_{k}"] = v
    save("selectors_16couples.npz", **d)

    geometry_fixtures()


if __name__ == "__main__":
    main()
