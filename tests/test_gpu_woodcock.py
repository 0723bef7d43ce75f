"""Woodcock gamma tracking in a layered box (hepem_woodcock_gamma).

Parity: the device kernel against the CPU port's restatement of the reference
helper's loop (G4HepEm/G4HepEm/src/G4HepEmWoodcockHelper.cc:146-299) over the
same box, on the same uniform streams: discrete outcomes identical, positions
and energies to 1e-12.  Physics: in a box of one material, Woodcock tracking
must give the same exponential interaction depths as ordinary tracking.
"""
import numpy as np
import pytest

from conftest import T3
from g4hepem_gb300 import workload as W

pytestmark = pytest.mark.gpu

NU = 32


def calorimeter(n_cells=50, pb=2.3, lar=5.7, half=200.0):
    """A sampling calorimeter of alternating G4_Pb (couple 2) and G4_lAr
    (couple 1) slabs along z; the Woodcock reference is Pb."""
    z = [0.0]
    imc = []
    for _ in range(n_cells):
        z += [z[-1] + pb, z[-1] + pb + lar]
        imc += [2, 1]
    return {"half_x": half, "half_y": half, "z_bounds": np.array(z), "layer_imc": np.array(imc, dtype=np.int32),
            "wdt_imc": 2, "energy_limit": 0.2}


def gammas_in_box(n, box, seed, emin=0.05, emax=1000.0):
    st = W.mixed_batch(n, n_couples=3, seed=seed, emin=emin, emax=emax, frac=(1.0, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    pos = (rng.uniform(-0.9, 0.9, n) * box["half_x"], rng.uniform(-0.9, 0.9, n) * box["half_y"],
           rng.uniform(box["z_bounds"][0], box["z_bounds"][-1], n))
    return st, pos


def gpu_woodcock(native, ctx, st, pos, box, seed):
    import torch
    n = len(st["ekin"])
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], NU, seed)
    p = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in pos)
    b = dict(box)
    b["z_bounds"] = torch.from_numpy(box["z_bounds"]).cuda()
    b["layer_imc"] = torch.from_numpy(box["layer_imc"]).cuda()
    reached = torch.zeros(n, dtype=torch.uint8, device="cuda")
    ctx.woodcock_gamma(sin, sout, p, b, u, NU, seed, res, reached)
    torch.cuda.synchronize()
    return native.to_numpy(sout), native.to_numpy(res), tuple(a.cpu().numpy() for a in p), reached.cpu().numpy()


def test_woodcock_matches_port(native, gpu_ctx, port):
    ctx = gpu_ctx(T3)
    box = calorimeter()
    n = 100000
    st, pos = gammas_in_box(n, box, seed=4)
    g_st, g_res, g_pos, g_reached = gpu_woodcock(native, ctx, st, pos, box, 12)
    pl = port(T3)
    u = pl.fill_uniforms(st["id"], NU, 12)
    p_st, p_res, p_pos, p_reached = pl.woodcock_gamma(st, pos, box, u, NU, 12)
    np.testing.assert_array_equal(g_reached, p_reached)
    for f in ("winner", "n_sec", "flags"):
        np.testing.assert_array_equal(g_res[f], p_res[f], err_msg=f)
    for f in ("imc", "rng_cursor", "gauss_valid"):
        np.testing.assert_array_equal(g_st[f], p_st[f], err_msg=f)
    for f in ("ekin", "nia0"):
        np.testing.assert_allclose(g_st[f], p_st[f], rtol=1e-12, atol=0, err_msg=f)
    for f in ("edep", "gstep"):
        np.testing.assert_allclose(g_res[f], p_res[f], rtol=1e-12, atol=0, err_msg=f)
    for a, b in zip(g_pos, p_pos):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12)
    for f in ("dir_x", "dir_y", "dir_z"):
        np.testing.assert_allclose(g_st[f], p_st[f], rtol=0, atol=1e-12, err_msg=f)
    ns = g_res["n_sec"].astype(int)
    valid = np.stack([ns > 0, ns > 1], axis=1).reshape(-1)
    np.testing.assert_allclose(g_res["sec_ekin"][valid], p_res["sec_ekin"][valid], rtol=1e-12)
    # both outcomes occur: interactions inside the box and boundary stops
    assert 0.05 < g_reached.mean() < 0.95
    assert np.all(g_res["gstep"] >= 0)
    # Woodcock-tracked gammas stay in the box (ordinary steps below the
    # energy limit are not limited by the geometry)
    wdt = st["ekin"] > box["energy_limit"]
    assert np.all(np.abs(g_pos[0][wdt]) <= box["half_x"]) and np.all(np.abs(g_pos[1][wdt]) <= box["half_y"])
    assert np.all((g_pos[2][wdt] >= box["z_bounds"][0]) & (g_pos[2][wdt] <= box["z_bounds"][-1]))


def test_woodcock_depth_distribution_in_one_material(native, gpu_ctx):
    # a box of Pb only: Woodcock tracking with the Pb reference is ordinary
    # tracking; the interaction depth of 10 MeV gammas is exponential with the
    # Pb mean free path
    import torch
    ctx = gpu_ctx(T3)
    box = {"half_x": 1e6, "half_y": 1e6, "z_bounds": np.array([0.0, 1e6]), "layer_imc": np.array([2], np.int32),
           "wdt_imc": 2, "energy_limit": 0.2}
    n = 400000
    st = W.fresh_state(np.full(n, 2), np.full(n, 2), np.full(n, 10.0), np.tile([[0.0, 0.0, 1.0]], (n, 1)),
                       np.full(n, 1.0))
    pos = (np.zeros(n), np.zeros(n), np.zeros(n))
    _, res, _, reached = gpu_woodcock(native, ctx, st, pos, box, 3)
    assert reached.sum() == 0
    # ordinary tracking of the same gammas: gstep = mfp * (-ln u)
    sin = native.state_to_torch(st)
    sout = native.empty_state_torch(n)
    r2 = native.alloc_out_torch(n)
    u = native.fill_uniforms(sin["id"], NU, 3)
    ctx.step(sin, sout, u, NU, 3, r2, form="plain")
    torch.cuda.synchronize()
    g = native.to_numpy(r2)["gstep"]
    mfp = float(np.mean(g))
    d = res["gstep"]
    # same stream, same first uniform: the Woodcock depth is the ordinary step
    np.testing.assert_allclose(d, g, rtol=1e-12)
    assert abs(d.mean() / mfp - 1) < 0.01
    assert abs(np.median(d) / (mfp * np.log(2)) - 1) < 0.02
