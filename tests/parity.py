"""Comparison of two step results (reference / oracle vs the GPU path).

Discrete outcomes must be identical: interaction chosen, number and type of
secondaries, flags, uniforms consumed (rejection-loop accept indices and the
target element show up there), Gauss-cache and MSC first-step state.
Continuous quantities must agree within RTOL = 1e-12 relative; direction
cosines, which pass through sin/cos of the host libm vs CUDA (<= 2 ulp), are
compared with an absolute 1e-12 (they are unit vectors), displacements
relative to their vector length.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-12

DISCRETE_STATE = ["rng_cursor", "gauss_valid", "msc_first_step"]
DISCRETE_RES = ["winner", "n_sec", "flags"]
CONT_STATE = ["ekin", "nia0", "nia1", "nia2", "nia3", "msc_init_range", "msc_dyn_factor", "msc_tlimit_min",
              "gauss_value"]
CONT_RES = ["edep", "gstep", "pstep"]


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    den = np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-300)
    r = np.abs(a - b) / den
    r[(a == b) | both_nan] = 0.0
    return r


def compare_steps(ref_state, ref_res, got_state, got_res, rtol=RTOL):
    """Return (report dict, ok).  Inputs are numpy dicts."""
    rep = {}
    ok = True
    n = len(ref_state["ekin"])
    for f in DISCRETE_STATE:
        bad = int(np.sum(ref_state[f] != got_state[f]))
        rep[f] = bad
        ok &= bad == 0
    for f in DISCRETE_RES:
        bad = int(np.sum(ref_res[f] != got_res[f]))
        rep[f] = bad
        ok &= bad == 0
    ns = ref_res["n_sec"].astype(int)
    slot_valid = (np.arange(2)[None, :] < ns[:, None]).reshape(-1)
    bad = int(np.sum((ref_res["sec_type"] != got_res["sec_type"]) & slot_valid))
    rep["sec_type"] = bad
    ok &= bad == 0
    gv = ref_state["gauss_valid"].astype(bool)
    for f in CONT_STATE:
        a, b = ref_state[f], got_state[f]
        if f == "gauss_value":
            a, b = a[gv], b[gv]
        r = _rel(a, b)
        rep[f] = float(r.max()) if r.size else 0.0
        ok &= rep[f] <= rtol
    for f in CONT_RES:
        r = _rel(ref_res[f], got_res[f])
        rep[f] = float(r.max()) if r.size else 0.0
        ok &= rep[f] <= rtol
    d = max(float(np.max(np.abs(ref_state[f"dir_{c}"] - got_state[f"dir_{c}"]))) for c in "xyz")
    rep["dir_abs"] = d
    ok &= d <= rtol
    dl = np.sqrt(sum(ref_res[f"disp_{c}"] ** 2 for c in "xyz"))
    dd = np.sqrt(sum((ref_res[f"disp_{c}"] - got_res[f"disp_{c}"]) ** 2 for c in "xyz"))
    m = dl > 0
    rep["disp_rel"] = float(np.max(dd[m] / dl[m])) if m.any() else 0.0
    ok &= rep["disp_rel"] <= rtol and bool(np.all(dd[~m] == 0))
    se = _rel(ref_res["sec_ekin"][slot_valid], got_res["sec_ekin"][slot_valid])
    rep["sec_ekin"] = float(se.max()) if se.size else 0.0
    ok &= rep["sec_ekin"] <= rtol
    sd = max(float(np.max(np.abs(ref_res[f"sec_dir_{c}"][slot_valid] - got_res[f"sec_dir_{c}"][slot_valid]),
                              initial=0.0)) for c in "xyz")
    rep["sec_dir_abs"] = sd
    ok &= sd <= rtol
    # exact-equality census (information only)
    rep["exact_ekin_frac"] = float(np.mean(ref_state["ekin"] == got_state["ekin"])) if n else 1.0
    return rep, bool(ok)


def energy_balance(state_in, state_out, res):
    """E_in (+2 m_e c^2 for an annihilating e+) - E_out - edep - sum(secondary E), per track."""
    mec2 = 0.51099890999999997
    n = len(state_in["ekin"])
    sec = res["sec_ekin"].reshape(n, 2)
    ns = res["n_sec"].astype(int)
    sec_sum = np.where(np.arange(2)[None, :] < ns[:, None], sec, 0.0).sum(1)
    stype = res["sec_type"].reshape(n, 2)
    # e+ annihilation (at rest or in flight) adds the rest masses; pair
    # production removes 2 m_e c^2 from the photon energy
    annih = (state_in["type"] == 1) & (ns == 2) & (stype[:, 0] == 2)
    pair = (state_in["type"] == 2) & (res["winner"] == 0) & (ns == 2)
    extra = np.where(annih, 2 * mec2, 0.0) - np.where(pair, 2 * mec2, 0.0)
    return state_in["ekin"] + extra - state_out["ekin"] - res["edep"] - sec_sum
