"""The multi-rank path of bench.py on the CPU (gloo, world size 2).

The stepping path shards by independent tracks: N ranks are N replicas, each
stepping its own disjoint range of track ids, with no collective on the data
path.  What is shared between ranks is the timing: a barrier around the timed
steps and the maximum of the per-rank times, from which the whole-job rate is
computed.  These tests run that host logic in two processes over gloo, and
the reference arm under torchrun, where rank 0 alone runs and prints.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["REPO"])
import numpy as np, torch, torch.distributed as dist
import bench
from g4hepem_gb300 import workload as W
ws, rank, _ = bench.dist_env()
dist.init_process_group("gloo", rank=rank, world_size=ws)
n = 1000
ids = W.mixed_batch(n, seed=bench.WORKLOAD_SEED, id0=bench.shard_id0(rank, n))["id"]
# rank r took 1 + 2 r seconds: the slowest replica sets the job time
t = bench.max_over_ranks(torch, 1.0 + 2.0 * rank, ws)
every = [None] * ws
dist.all_gather_object(every, [int(x) for x in ids])
dist.barrier()
print(json.dumps({"rank": rank, "t": t, "ids": every, "rate": bench.whole_job_rate(ws, n, 5, t)}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replicas_step_disjoint_shards_and_time_on_the_slowest_rank():
    ws, port = 2, _free_port()
    procs = []
    for rank in range(ws):
        env = dict(os.environ, REPO=REPO, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], cwd=REPO, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=240)
            assert p.returncode == 0, err[-2000:]
            outs.append(json.loads(out.strip().splitlines()[-1]))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    n = 1000
    for o in outs:
        assert o["t"] == 3.0
        assert o["rate"] == pytest.approx(ws * n * 5 / 3.0)
        shards = [set(x) for x in o["ids"]]
        assert all(len(s) == n for s in shards)
        assert not (shards[0] & shards[1])
        assert shards[0] | shards[1] == set(range(ws * n))


def test_reference_arm_under_torchrun_prints_once_from_rank_0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--tracks", "4096", "--steps", "1", "--warmup", "1"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["unit"] == "steps/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
