"""One geometry-limited step through the compiled C++ client
(tests/client/hepem_client.cpp: ElectronManager::HowFar, the transport,
GammaManager::Perform of include/g4hepem_gb300.hh), compared with the
reference's golden results (discrete identical, continuous within 1e-12) and
with the CPU port on the same inputs."""
import os
import subprocess

import numpy as np
import pytest

from client_build import build_client
from conftest import T3, golden_res, golden_state, load_golden
from g4hepem_gb300 import workload as W
from g4hepem_gb300.native import OUT_FIELDS, STATE_FIELDS
from parity import compare_steps

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", ["plain", "batched"])
def test_cpp_client_geometry_step(native, gpu_ctx, port, tmp_path, form):
    gpu_ctx(T3)  # skips without a GPU
    exe = build_client()
    g = load_golden("geosteps_3couples.npz")
    seed = int(g["seed"][0])
    st = golden_state(g, "g1_", "in")
    for f, dt in STATE_FIELDS:
        np.ascontiguousarray(st[f], dtype=dt).tofile(os.path.join(tmp_path, f"in_{f}.bin"))
    for key in ("gfrac", "ndir_x", "ndir_y", "ndir_z", "post_bnd"):
        np.ascontiguousarray(g[f"g1_{key}"]).tofile(os.path.join(tmp_path, f"{key}.bin"))
    r = subprocess.run([exe, "step", T3, str(tmp_path), form, str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    n = len(st["ekin"])
    out = {f: np.fromfile(os.path.join(tmp_path, f"out_{f}.bin"), dtype=dt) for f, dt in STATE_FIELDS}
    res = {f: np.fromfile(os.path.join(tmp_path, f"res_{f}.bin"), dtype=dt) for f, dt, _ in OUT_FIELDS}
    proposed = np.fromfile(os.path.join(tmp_path, "proposed.bin"), dtype=np.float64)
    assert len(proposed) == n and np.array_equal(proposed, g["g1_proposed"])
    ref_out, ref_res = golden_state(g, "g1_", "out"), golden_res(g, "g1_")
    rep, ok = compare_steps(ref_out, ref_res, out, res)
    assert ok, rep
    # the CPU port on the same inputs
    nd = (g["g1_ndir_x"], g["g1_ndir_y"], g["g1_ndir_z"])
    u = W.philox_uniforms(seed, st["id"], 64)
    p_out, p_res, _ = port(T3).step_geom(st, u, 64, seed, g["g1_gfrac"], nd, g["g1_post_bnd"])
    rep, ok = compare_steps(p_out, p_res, out, res)
    assert ok, rep
