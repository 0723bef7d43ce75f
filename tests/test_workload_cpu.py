"""The synthetic workloads that stand in for the reference's benchmark inputs
have the shapes, sizes and distributions the measurements are quoted on.

* the 4M-track step: 45% gamma, 45% e-, 10% e+, kinetic energies log-uniform
  in [1 MeV, 10 GeV], couples uniform, isotropic unit directions, tracks at
  their first step (the reset state of G4HepEmTrack / G4HepEmMSCTrackData);
* the electron lookups: e- log-uniform in [1 keV, 100 TeV];
* the batching workload: 64 log-normal sub-batch sizes clipped to [1k, 1M]
  that sum to 16,777,216 tracks;
* the uniform streams: Philox4x32-10 per (seed, track id), independent of the
  batch a track sits in.
"""
import numpy as np

from g4hepem_gb300 import workload as W


def test_mixed_step_batch_has_the_stated_mix_and_ranges():
    n = 1 << 20
    st = W.mixed_batch(n, seed=7)
    frac = np.bincount(st["type"].astype(np.int64), minlength=3) / n
    # type 0 e-, 1 e+, 2 gamma
    assert abs(frac[2] - 0.45) < 0.003 and abs(frac[0] - 0.45) < 0.003 and abs(frac[1] - 0.10) < 0.002
    e = st["ekin"]
    assert e.min() >= 1.0 and e.max() <= 1.0e4
    le = np.log(e)
    # log-uniform: mean and spread of log E of a uniform on [0, ln 1e4]
    assert abs(le.mean() - 0.5 * np.log(1e4)) < 0.01
    assert abs(le.std() - np.log(1e4) / np.sqrt(12.0)) < 0.01
    assert np.all(np.bincount(st["imc"].astype(np.int64), minlength=3) > n // 3 - 3000)
    norm = st["dir_x"] ** 2 + st["dir_y"] ** 2 + st["dir_z"] ** 2
    assert np.allclose(norm, 1.0, rtol=0, atol=1e-12)
    assert abs(st["dir_z"].mean()) < 0.01
    # first step: the reset state of the reference's track types
    for k in ("nia0", "nia1", "nia2", "nia3"):
        assert np.all(st[k] == -1.0)
    assert np.all(st["msc_init_range"] == 1e21) and np.all(st["msc_dyn_factor"] == 0.04)
    assert np.all(st["msc_tlimit_min"] == 1e-7) and np.all(st["msc_first_step"] == 1)
    assert np.all(st["gauss_valid"] == 0) and np.all(st["rng_cursor"] == 0)
    assert np.all(st["on_boundary"] == 0) and np.all(st["safety"] > 0)


def test_rank_shards_are_the_same_tracks_with_disjoint_ids():
    a = W.mixed_batch(1000, seed=7, id0=0)
    b = W.mixed_batch(1000, seed=7, id0=1000)
    assert np.array_equal(a["id"], np.arange(1000)) and np.array_equal(b["id"], np.arange(1000, 2000))
    assert np.array_equal(a["ekin"], b["ekin"])


def test_electron_lookup_batch_ranges():
    e, imc = W.electron_lookup_batch(1 << 16, seed=11)
    assert e.min() >= 1e-3 and e.max() <= 1e8
    assert set(np.unique(imc)) == {0, 1, 2}


def test_subbatch_sizes_sum_clip_and_median():
    s, sigma = W.subbatch_sizes()
    assert len(s) == 64 and int(s.sum()) == 1 << 24
    assert s.min() >= 1000 and s.max() <= 1 << 20
    assert len(np.unique(s)) > 16  # uneven
    # the median of the draws is the stated 30k (no rescaling of the sizes)
    assert 0.5 * 30000 < np.median(s) < 2.0 * 30000
    assert 2.0 < sigma < 8.0


def test_uniform_streams_depend_on_seed_and_id_only():
    ids = np.array([5, 7, 11], dtype=np.int32)
    u = W.philox_uniforms(99, ids, 8)
    u_sub = W.philox_uniforms(99, ids[1:], 8)
    assert np.array_equal(u[1:], u_sub)
    assert np.all((u > 0.0) & (u < 1.0))
    assert not np.array_equal(u, W.philox_uniforms(100, ids, 8))
