"""Synthetic track batches of the benchmark configurations.

Tracks are drawn from a seeded numpy Philox generator; the per-track uniform
streams follow the contract of include/g4hepem_gb300.h (Philox4x32-10 with
counter (k>>1, id, 0, 0x48455045) and key = seed), vectorised here so that
host-side tests can build streams without a GPU.
"""
from __future__ import annotations

import numpy as np

TYPE_EM, TYPE_EP, TYPE_GAMMA = 0, 1, 2

STATE_DTYPES = dict(type=np.int8, imc=np.int32, id=np.int32, ekin=np.float64, dir_x=np.float64,
                    dir_y=np.float64, dir_z=np.float64, nia0=np.float64, nia1=np.float64, nia2=np.float64,
                    nia3=np.float64, safety=np.float64, on_boundary=np.uint8, msc_init_range=np.float64,
                    msc_dyn_factor=np.float64, msc_tlimit_min=np.float64, msc_first_step=np.uint8,
                    gauss_valid=np.uint8, gauss_value=np.float64, rng_cursor=np.int32)
STATE_FIELDS = list(STATE_DTYPES)

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
_MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 (Salmon et al., SC'11) over uint32 arrays."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint32) for x in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & _MASK32).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & _MASK32).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + _W0)
            k1 = np.uint32(k1 + _W1)
    return c0, c1, c2, c3


def philox_uniforms(seed: int, ids: np.ndarray, n_uniform: int, k0: int = 0) -> np.ndarray:
    """uniforms[i, k] = stream value k0+k of track ids[i]; shape (n, n_uniform)."""
    ids = np.asarray(ids, dtype=np.int64).astype(np.uint32)
    ks = np.arange(k0, k0 + n_uniform, dtype=np.int64)
    kk = np.broadcast_to(ks[None, :], (len(ids), n_uniform))
    ii = np.broadcast_to(ids[:, None], (len(ids), n_uniform))
    r0, r1, r2, r3 = philox4x32_10((kk >> 1).astype(np.uint32), ii, np.zeros_like(ii, dtype=np.uint32),
                                   np.full(ii.shape, 0x48455045, dtype=np.uint32),
                                   seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    odd = (kk & 1).astype(bool)
    a = np.where(odd, r2, r0).astype(np.uint64)
    b = np.where(odd, r3, r1).astype(np.uint64)
    bits = (a << np.uint64(20)) | (b >> np.uint64(12))
    return (bits.astype(np.float64) + 0.5) * (1.0 / 4503599627370496.0)


def fresh_state(types, imc, ekin, dirs, safety, ids=None, on_boundary=None) -> dict:
    """Track-state arrays of tracks at their first step (reset MSC and RNG state,
    G4HepEmTrack / G4HepEmMSCTrackData ReSet values)."""
    n = len(types)
    st = {}
    st["type"] = np.asarray(types, dtype=np.int8).copy()
    st["imc"] = np.asarray(imc, dtype=np.int32).copy()
    st["id"] = (np.arange(n, dtype=np.int32) if ids is None else np.asarray(ids, dtype=np.int32).copy())
    st["ekin"] = np.asarray(ekin, dtype=np.float64).copy()
    st["dir_x"] = np.ascontiguousarray(dirs[:, 0], dtype=np.float64)
    st["dir_y"] = np.ascontiguousarray(dirs[:, 1], dtype=np.float64)
    st["dir_z"] = np.ascontiguousarray(dirs[:, 2], dtype=np.float64)
    for k in ("nia0", "nia1", "nia2", "nia3"):
        st[k] = np.full(n, -1.0)
    st["safety"] = np.asarray(safety, dtype=np.float64).copy()
    st["on_boundary"] = (np.zeros(n, dtype=np.uint8) if on_boundary is None
                         else np.asarray(on_boundary, dtype=np.uint8).copy())
    st["msc_init_range"] = np.full(n, 1.0e21)
    st["msc_dyn_factor"] = np.full(n, 0.04)
    st["msc_tlimit_min"] = np.full(n, 1.0e-7)
    st["msc_first_step"] = np.ones(n, dtype=np.uint8)
    st["gauss_valid"] = np.zeros(n, dtype=np.uint8)
    st["gauss_value"] = np.zeros(n)
    st["rng_cursor"] = np.zeros(n, dtype=np.int32)
    return st


def isotropic(rng, n):
    cost = 2.0 * rng.random(n) - 1.0
    phi = 2.0 * np.pi * rng.random(n)
    sint = np.sqrt((1.0 - cost) * (1.0 + cost))
    d = np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=1)
    return d / np.linalg.norm(d, axis=1)[:, None]


def mixed_batch(n: int, n_couples: int = 3, seed: int = 7, emin=1.0, emax=1.0e4,
                frac=(0.45, 0.45, 0.10), safety_range=(1e-4, 10.0), id0: int = 0) -> dict:
    """Mixed gamma / e- / e+ batch: energies log-uniform in [emin, emax] MeV,
    couples uniform, isotropic directions, safety log-uniform (mm), first step."""
    rng = np.random.Generator(np.random.Philox(seed))
    u = rng.random(n)
    types = np.where(u < frac[0], TYPE_GAMMA, np.where(u < frac[0] + frac[1], TYPE_EM, TYPE_EP))
    ekin = np.exp(np.log(emin) + (np.log(emax) - np.log(emin)) * rng.random(n))
    imc = rng.integers(0, n_couples, size=n)
    dirs = isotropic(rng, n)
    lo, hi = np.log(safety_range[0]), np.log(safety_range[1])
    safety = np.exp(lo + (hi - lo) * rng.random(n))
    return fresh_state(types, imc, ekin, dirs, safety, ids=np.arange(id0, id0 + n, dtype=np.int32))


def transport(state: dict, seed: int, f_short=0.45, f_tiny=0.08, f_zero=0.02, f_turn=0.3):
    """What a caller's geometry does to a batch between HowFar and Perform.

    Returns (gfrac, new_dir, post_boundary): per track the fraction of the
    proposed geometrical step that transport makes (1: the proposed step; a
    shortened step: uniform in (0.05, 1) with probability f_short, log-uniform
    in [1e-7, 1e-2] with probability f_tiny, 0 with probability f_zero), the
    direction after transport (e+-: a fraction f_turn turned by up to 0.2 rad,
    as a magnetic field does; gammas keep theirs), and the post-step boundary
    status (80% of the shortened steps end on a boundary, 5% of the others)."""
    n = len(state["ekin"])
    rng = np.random.Generator(np.random.Philox(seed))
    u = rng.random(n)
    gfrac = np.ones(n)
    short = u < f_short
    gfrac[short] = 0.05 + 0.95 * rng.random(int(short.sum()))
    tiny = (u >= f_short) & (u < f_short + f_tiny)
    gfrac[tiny] = np.exp(np.log(1e-7) + (np.log(1e-2) - np.log(1e-7)) * rng.random(int(tiny.sum())))
    gfrac[(u >= f_short + f_tiny) & (u < f_short + f_tiny + f_zero)] = 0.0
    shortened = gfrac < 1.0
    post = np.where(shortened, rng.random(n) < 0.8, rng.random(n) < 0.05).astype(np.uint8)
    d = np.stack([state["dir_x"], state["dir_y"], state["dir_z"]], axis=1).copy()
    turn = (state["type"] != TYPE_GAMMA) & (rng.random(n) < f_turn)
    k = int(turn.sum())
    if k:
        axis = isotropic(rng, k)
        ang = 0.2 * rng.random(k)
        v = d[turn]
        # Rodrigues rotation of v about axis by ang, renormalised
        c, s = np.cos(ang)[:, None], np.sin(ang)[:, None]
        kv = np.cross(axis, v)
        kd = np.sum(axis * v, axis=1)[:, None]
        w = v * c + kv * s + axis * kd * (1.0 - c)
        d[turn] = w / np.linalg.norm(w, axis=1)[:, None]
    new_dir = tuple(np.ascontiguousarray(d[:, j]) for j in range(3))
    return gfrac, new_dir, post


def electron_lookup_batch(n: int, n_couples: int = 3, seed: int = 11, emin=1e-3, emax=1e8):
    """e- energies log-uniform in [1 keV, 100 TeV] and uniform couples."""
    rng = np.random.Generator(np.random.Philox(seed))
    ekin = np.exp(np.log(emin) + (np.log(emax) - np.log(emin)) * rng.random(n))
    imc = rng.integers(0, n_couples, size=n).astype(np.int32)
    return ekin, imc


def subbatch_sizes(total: int = 1 << 24, n_sub: int = 64, median: float = 30000.0, lo: int = 1000,
                   hi: int = 1 << 20, seed: int = 3):
    """Uneven sub-batch sizes of the batching workload: log-normal with the
    given median, clipped to [lo, hi], with the width sigma chosen so that the
    clipped sizes of the n_sub draws sum to `total` (the draws z_k of a
    standard normal are fixed by the seed, sigma is found by bisection on the
    clipped sum of median * exp(sigma z_k), with the z_k shifted so that their
    median is 0; rounding is absorbed by the sizes inside the clip range).
    Returns (sizes, sigma)."""
    rng = np.random.Generator(np.random.Philox(seed))
    z = rng.standard_normal(n_sub)
    z -= np.median(z)  # the median draw is the stated median

    def clipped_sum(sig):
        return np.clip(median * np.exp(sig * z), lo, hi).sum()

    s_lo, s_hi = 0.0, 20.0
    for _ in range(200):
        sig = 0.5 * (s_lo + s_hi)
        if clipped_sum(sig) < total:
            s_lo = sig
        else:
            s_hi = sig
    sigma = 0.5 * (s_lo + s_hi)
    sizes = np.clip(np.round(median * np.exp(sigma * z)), lo, hi).astype(np.int64)
    diff = total - int(sizes.sum())
    free = [k for k in np.argsort(-sizes) if lo < sizes[k] < hi]
    k = 0
    while diff != 0 and free:
        j = free[k % len(free)]
        step = int(np.clip(sizes[j] + diff, lo, hi)) - int(sizes[j])
        sizes[j] += step
        diff -= step
        k += 1
        if k > 10 * n_sub:
            break
    return sizes, sigma
