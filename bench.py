"""Benchmark of the G4HepEmRun stepping-physics path on GB300.

Workload (the 4M mixed-track step): 4,194,304 tracks, 45% gamma / 45% e- /
10% e+, kinetic energies log-uniform in [1 MeV, 10 GeV], couples uniform over
G4_PbWO4 / G4_lAr / G4_Pb at 0.7 mm (synthetic G4HepEmState tables), isotropic
directions, first-step track state, 64 Philox uniforms per track.  One "step"
= one HowFar + Perform of every track.  `--form mixed` (default) steps it with
the precision form (hepem_step_mixed: FP32 bulk, FP64 where the error budget
needs it, discrete outcomes identical to the FP64 path); `--form batched` with
the FP64 batched form (bit-exact with the reference CPU functions).  The plain
FP64 form (hepem_step, bit-exact) is timed beside either.  Each timed step reads the same input state and
writes separate outputs, so every step does identical work; the inputs
(~2.7 GB) are larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput
(steps/s over all ranks); `e2e` is the same metric through the host-buffer
C-ABI entry point of the form (hepem_step_host_mixed, or hepem_step_host for
--form batched) with the host<->device copies of the track state inside the
timed region (the uniforms are drawn on the device from the
same counter-based stream, n_uniform = 0).  `--impl reference` times the reference algorithm on the host
cores: the CPU port of the oracle (the reference build needs the reference
sources, which only the development host has), all host threads, same workload
and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

TABLE = os.path.join(REPO, "g4hepem_gb300", "data", "three_couples_0.7mm.json")
N_TRACKS = 4194304
NU = 64
SEED = 20261203
WORKLOAD_SEED = 7
LAUNCHES_PER_STEP = 14  # 3 sort kernels, 2 stage-A kernels, 9 interaction kernels (plus two memsets)
# precision form: + one FP64 fallback kernel at the end of the step
LAUNCHES_PER_STEP_MIXED = 15
METRIC = "mixed e±/γ physics steps/s (1 GB300) vs plain FP64 path; p50/p99 batch latency"
UNIT = "steps/s"
CONFIG = {"workload": "full physics step (HowFar + Perform), 4,194,304 mixed tracks (45% gamma, 45% e-, 10% e+), "
                      "1 MeV-10 GeV log-uniform, 3 couples (G4_PbWO4, G4_lAr, G4_Pb @0.7 mm), "
                      "64 Philox uniforms/track",
          "tracks_per_step": N_TRACKS, "uniforms_per_track": NU, "table": "three_couples_0.7mm.json",
          "l2": "inputs larger than L2 (2.7 GB per step), no flush"}


def shard_id0(rank: int, n: int) -> int:
    """First track id of a rank's batch: ranks step disjoint id ranges of
    independent tracks (replicas; no collective on the data path)."""
    return rank * n


def max_over_ranks(torch, value: float, ws: int) -> float:
    """The largest per-rank time: the slowest replica sets the whole-job time
    (on the device of the process group's backend: CUDA for NCCL)."""
    if ws <= 1:
        return value
    dist = torch.distributed
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ws: int, n: int, steps: int, seconds: float) -> float:
    """Steps/s of all ranks together: every rank steps n tracks per step."""
    return ws * n * steps / seconds


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(n, uniforms_consumed, secondaries):
    """Bytes of the C-ABI contract fields read and written once per step.

    read : full input state, 128 B/track (type 1, imc 4, id 4, ekin 8, dir 24,
           nia 32, safety 8, boundary 1, MSC 25, Gauss 9, cursor 4) plus the
           uniforms actually consumed (8 B each);
    write: persistent state 102 B/track (ekin, dir, nia, MSC, Gauss, cursor),
           step results 51 B/track (edep, gstep, pstep, winner, disp, flags,
           n_sec) and 33 B per secondary produced (type, E, dir)."""
    return n * (128 + 102 + 51) + 8 * uniforms_consumed + 33 * secondaries


def fp64_peak_tflops(torch):
    """Measured FP64 peak of this GPU: cuBLAS DGEMM 4096^3, best of 5."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * 4096 ** 3 / best / 1e12


def host_link_gbs(torch):
    """Measured host<->device bandwidth: concurrent pinned H2D and D2H copies of
    2 GiB each on two streams (bytes of both directions / time), best of 3."""
    n = 1 << 28
    h1 = torch.empty(n, dtype=torch.float64).pin_memory()
    h2 = torch.empty(n, dtype=torch.float64).pin_memory()
    d1 = torch.empty(n, dtype=torch.float64, device="cuda")
    d2 = torch.empty(n, dtype=torch.float64, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    best = 1e30
    for _ in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s1):
            d1.copy_(h1, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    del h1, h2, d1, d2
    return 16 * n / best / 1e9


def fp32_peak_tflops(torch):
    """Measured FP32 (SIMT) peak of this GPU: cuBLAS SGEMM 8192^3 with TF32 off, best of 5."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
        b = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            a @ b
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e) / 1e3)
        return 2 * 8192 ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def profile_summary(name):
    p = os.path.join(REPO, "profiles", name)
    try:
        return json.load(open(p))
    except Exception:
        return None


def c1_lookups(torch, N, ctx, stream, args, hbm):
    """Electron lookups: 2^20 e- with energies log-uniform in
    [1 keV, 100 TeV] over the 3 couples; restricted ionisation and brem cross
    sections, dE/dx, range and inverse range at half the range per track
    (hepem_electron_lookup).  Inputs 12 B + outputs 40 B per track; the
    2^20-track batch (54.5 MB) fits L2, so each timed launch reads a fresh
    batch slice of a 16x larger buffer (inputs larger than L2)."""
    from g4hepem_gb300 import workload as W
    n1, reps = 1 << 20, 16
    e_np, i_np = W.electron_lookup_batch(n1 * reps, seed=11)
    ekin = torch.from_numpy(e_np).cuda()
    imc = torch.from_numpy(i_np).cuda()
    outs = [{k: torch.empty(n1, dtype=torch.float64, device="cuda")
             for k in ("xs_ioni", "xs_brem", "dedx", "range", "invrange_half")} for _ in range(2)]
    for r in range(3):
        ctx.electron_lookup(ekin[r * n1:(r + 1) * n1], imc[r * n1:(r + 1) * n1], out=outs[r % 2], stream=stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = max(args.steps, reps)
    ev0.record(stream)
    for r in range(k):
        s = (r % reps) * n1
        ctx.electron_lookup(ekin[s:s + n1], imc[s:s + n1], out=outs[r % 2], stream=stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / k
    alg = n1 * (8 + 4 + 5 * 8)
    return {"workload": "2^20 e-, 1 keV-100 TeV log-uniform, 3 couples, 5 lookups per track",
            "value": n1 / (ms / 1e3), "unit": "tracks/s", "ms_per_launch": ms, "launches": k,
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": alg / (ms / 1e3) / 1e9 / hbm, "algorithmic_bytes_per_launch": alg,
                         "note": "FP64-issue bound like the step (VDT log, 4 splines, range bisection)"}}


def c3_batching(torch, N, args):
    """Uneven batching: 64 sub-batches of log-normal sizes (median 30k,
    clipped to [1k, 1M], the width fitted so that the sizes sum to 16,777,216
    tracks), the particle and energy mix of the 4M-track step, 16 random couples
    (1-4 elements, Z in 1..82, 1-12 g/cm3, cuts 0.1/0.7/1.0 mm).  Timed: one
    call per sub-batch with the plain form, the batched form with the default
    launch configuration and with the configuration chosen by the autotuner
    (also captured once in a CUDA graph and replayed), the precision form
    (called and replayed from a graph); and all sub-batches in one
    hepem_step_subbatches call, in the batched and the precision form (these
    with the default launch configuration)."""
    from g4hepem_gb300 import workload as W
    table = os.path.join(REPO, "g4hepem_gb300", "data", "random16.json")
    ctx = N.Context(table)
    sizes, sigma = W.subbatch_sizes()
    total = int(sizes.sum())
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    st = W.mixed_batch(total, n_couples=16, seed=17)
    sin = N.state_to_torch(st)
    sout = N.empty_state_torch(total)
    res = N.alloc_out_torch(total)
    u = N.fill_uniforms(sin["id"], NU, SEED)
    slots = {f: k for f, _, k in N.OUT_FIELDS}

    def one_pass(form):
        for b in range(len(sizes)):
            a, e = int(off[b]), int(off[b + 1])
            ctx.step({k: v[a:e] for k, v in sin.items()}, {k: v[a:e] for k, v in sout.items()},
                     u[a * NU:e * NU], NU, SEED, {k: v[a * slots[k]:e * slots[k]] for k, v in res.items()},
                     form=form)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(reps):
            fn()
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    reps = max(2, min(args.steps, 5))
    ms_plain = timed(lambda: one_pass("plain"), 1)
    ms_default = timed(lambda: one_pass("batched"), reps)
    # launch configuration chosen by the autotuner on a 2^20-track sample of the workload
    ns = 1 << 20
    tuned = ctx.autotune({k: v[:ns] for k, v in sin.items()}, u[:ns * NU], NU, SEED, apply=True)
    ms_batched = timed(lambda: one_pass("batched"), reps)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        one_pass("batched")
    torch.cuda.current_stream().wait_stream(side)
    with torch.cuda.graph(graph):
        one_pass("batched")
    ms_graph = timed(graph.replay, reps)
    # the precision form and the one-call passes with the default launch
    # configuration (the tuner times the FP64 form's kernels)
    ctx.set_launch_config(None)
    # the same sub-batches through the precision form, also captured and replayed
    ms_mixed = timed(lambda: one_pass("mixed"), reps)
    graph_m = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        one_pass("mixed")
    torch.cuda.current_stream().wait_stream(side)
    with torch.cuda.graph(graph_m):
        one_pass("mixed")
    ms_mixed_graph = timed(graph_m.replay, reps)
    # all 64 sub-batches in one sorted, queued pass (hepem_step_subbatches)
    batches = [(int(off[b]), int(sizes[b]), SEED) for b in range(len(sizes))]
    ms_sub = timed(lambda: ctx.step_subbatches(batches, sin, sout, u, NU, res, form="batched"), reps)
    ms_sub_mixed = timed(lambda: ctx.step_subbatches(batches, sin, sout, u, NU, res, form="mixed"), reps)
    ctx.close()
    return {"workload": f"64 sub-batches (log-normal, median 30k, sigma {sigma:.2f} fitted so that the sizes "
                        "clipped to [1k, 1M] sum to 16,777,216 tracks), 16 random couples, the particle/energy "
                        "mix of the 4M-track step",
            "subbatch_min": int(sizes.min()), "subbatch_median": float(np.median(sizes)),
            "subbatch_max": int(sizes.max()), "subbatch_sigma": sigma,
            "batched_subbatches": {"value": total / (ms_sub / 1e3), "unit": UNIT, "ms_per_pass": ms_sub,
                                   "entry_point": "hepem_step_subbatches (HEPEM_FORM_BATCHED), one call"},
            "mixed_subbatches": {"value": total / (ms_sub_mixed / 1e3), "unit": UNIT, "ms_per_pass": ms_sub_mixed,
                                 "entry_point": "hepem_step_subbatches (HEPEM_FORM_MIXED), one call"},
            "plain": {"value": total / (ms_plain / 1e3), "unit": UNIT, "ms_per_pass": ms_plain},
            "batched_default_launch": {"value": total / (ms_default / 1e3), "unit": UNIT, "ms_per_pass": ms_default},
            "batched": {"value": total / (ms_batched / 1e3), "unit": UNIT, "ms_per_pass": ms_batched,
                        "launch": "autotuned (hepem_autotune on 2^20 tracks)"},
            "autotuned_config": tuned,
            "batched_graph": {"value": total / (ms_graph / 1e3), "unit": UNIT, "ms_per_pass": ms_graph,
                              "launches_per_pass": LAUNCHES_PER_STEP * len(sizes)},
            "vs_plain": ms_plain / ms_graph,
            "mixed": {"value": total / (ms_mixed / 1e3), "unit": UNIT, "ms_per_pass": ms_mixed,
                      "entry_point": "hepem_step_mixed"},
            "mixed_graph": {"value": total / (ms_mixed_graph / 1e3), "unit": UNIT, "ms_per_pass": ms_mixed_graph,
                            "launches_per_pass": LAUNCHES_PER_STEP_MIXED * len(sizes)},
            "mixed_vs_plain": ms_plain / ms_mixed_graph}


def f_rows(torch, N, ctx, sout, res, hbm):
    """The rows after the step: secondary stacking with production cuts on the
    4M-track step's own results (hepem_stack_secondaries), and Woodcock γ
    tracking of 2^22 γ in a 50-cell Pb / lAr sampling calorimeter
    (hepem_woodcock_gamma), each timed with CUDA events around the call."""
    def timed(fn, reps=5, before=None):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            if before:
                before()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    n = sout["ekin"].numel()
    out = N.empty_state_torch(2 * n)
    edep = torch.zeros(n, dtype=torch.float64, device="cuda")
    holder = {}

    def stack():
        holder["r"] = ctx.stack_secondaries(sout, res, True, 1 << 30, 2 * n, out=out, edep_cut=edep)
    ms_stack = timed(stack)
    n_stacked = int(holder["r"][1].item())
    n_sec = int(res["n_sec"].to(torch.int64).sum().item())
    # algorithmic bytes: per parent its secondary count, couple and safety; per
    # secondary its slot (type, energy, direction); per stacked track a full state
    alg = n * (1 + 4 + 8) + n_sec * 33 + n_stacked * 120 + n * 8
    stacking = {"workload": "the secondaries of one 4,194,304-track precision-form step, production cuts applied",
                "parents": n, "secondaries": n_sec, "stacked": n_stacked, "ms_per_call": ms_stack,
                "value": n / (ms_stack / 1e3), "unit": "parent tracks/s",
                "roofline": {"bound": "hbm", "achieved": alg / (ms_stack / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                             "frac": alg / (ms_stack / 1e3) / 1e9 / hbm, "algorithmic_bytes_per_call": alg}}

    from g4hepem_gb300 import workload as W
    ng = 1 << 22
    z = [0.0]
    imc = []
    for _ in range(50):
        z += [z[-1] + 2.3, z[-1] + 2.3 + 5.7]
        imc += [2, 1]
    st = W.mixed_batch(ng, n_couples=3, seed=23, emin=0.05, emax=1000.0, frac=(1.0, 0.0, 0.0))
    rng = np.random.default_rng(23)
    pos0 = [torch.from_numpy(a).cuda() for a in (rng.uniform(-180.0, 180.0, ng), rng.uniform(-180.0, 180.0, ng),
                                                 rng.uniform(0.0, z[-1], ng))]
    pos = [a.clone() for a in pos0]
    box = {"half_x": 200.0, "half_y": 200.0, "z_bounds": torch.tensor(z, dtype=torch.float64, device="cuda"),
           "layer_imc": torch.tensor(imc, dtype=torch.int32, device="cuda"), "wdt_imc": 2, "energy_limit": 0.2}
    gin = N.state_to_torch(st)
    gout = N.empty_state_torch(ng)
    gres = N.alloc_out_torch(ng)
    u = N.fill_uniforms(gin["id"], 32, SEED)
    reached = torch.zeros(ng, dtype=torch.uint8, device="cuda")

    def reset():
        for a, b in zip(pos, pos0):
            a.copy_(b)
        reached.zero_()
    ms_wdt = timed(lambda: ctx.woodcock_gamma(gin, gout, tuple(pos), box, u, 32, SEED, gres, reached),
                   before=reset)
    woodcock = {"workload": "4,194,304 γ, 50 keV-1 GeV log-uniform, in a 50-cell G4_Pb / G4_lAr calorimeter "
                            "(2.3 / 5.7 mm slabs, Pb the Woodcock reference), 32 uniforms per track",
                "ms_per_call": ms_wdt, "value": ng / (ms_wdt / 1e3), "unit": "γ tracks/s (to an interaction or "
                "out of the box)", "reached_interaction": int(reached.sum().item())}
    return {"stacking": stacking, "woodcock": woodcock}


def c4_serving(torch, N, args):
    """Serving: an event stream through the serving form
    (hepem_server_*).  A request is one event's track batch, log-normal in size
    (median 2k tracks, sigma 1.5, clipped to [1, 500k]), with the
    particle / energy / couple mix of the 4M-track step; 256 distinct event batches
    are drawn once and re-submitted with fresh seeds (new uniform streams).
    Memory admission budget 16 GB; tracks stay resident until they fall below
    1 keV or the request reaches 1000 steps.  First the sustained peak: a
    closed loop with 512 requests in flight; then open-loop Poisson arrivals at
    25/50/90% of that peak request rate.  Reported per level: steps/s, p50/p99 request
    latency (submit to result) and p50/p99 batch latency (one server
    iteration: one batched step over every resident track).  The server steps
    in the form of the headline (--form: the precision form by default)."""
    from g4hepem_gb300 import workload as W
    ctx = N.Context(TABLE)
    # the server steps in the bench's form (precision form by default)
    srv = N.Server(ctx, memory_budget_bytes=16 << 30, max_steps=1000, max_requests=4096, min_energy=1.0e-3,
                   mixed=args.form == "mixed")
    rng = np.random.Generator(np.random.Philox(41))
    sizes = np.clip(np.round(2000.0 * np.exp(1.5 * rng.standard_normal(256))), 1, 500000).astype(np.int64)
    events = [W.mixed_batch(int(m), seed=1000 + k) for k, m in enumerate(sizes)]
    seed_next = [1 << 40]

    def submit(k):
        seed_next[0] += 1
        return srv.submit(events[k % len(events)], seed=seed_next[0])

    def collect(ids):
        return [srv.wait(i, timeout_s=300.0)[0] for i in ids]

    def summary(res, t_first, st):
        t_end = max(r["t_done"] for r in res)
        window = t_end - t_first
        lat = np.array([r["t_done"] - r["t_submit"] for r in res]) * 1e3
        steps = sum(r["track_steps"] for r in res)
        return {"requests": len(res), "tracks": int(sum(r["n_tracks"] for r in res)),
                "track_steps": int(steps), "seconds": window, "steps_per_s": steps / window,
                "requests_per_s": len(res) / window,
                "request_ms_p50": float(np.percentile(lat, 50)), "request_ms_p99": float(np.percentile(lat, 99)),
                "batch_ms_p50": st["batch_ms_p50"], "batch_ms_p99": st["batch_ms_p99"],
                "iterations": st["iterations"], "mean_tracks_per_iteration": st["track_steps"] / max(1, st["iterations"])}

    # warm-up, then the sustained peak: a closed loop that keeps 512 requests
    # in flight for 3 s (each completion is replaced by a new request); the
    # rates are read over the last 2 s from the server's own counters
    collect([submit(k) for k in range(64)])
    inflight, k = [], 0
    for _ in range(512):
        inflight.append(submit(k))
        k += 1
    t_start = time.monotonic()
    measuring = False
    done_in_window = []
    while time.monotonic() - t_start < 3.0:
        r = srv.wait(inflight.pop(0), timeout_s=300.0)[0]
        if not measuring and time.monotonic() - t_start > 1.0:
            srv.reset_stats()
            measuring, t_win = True, time.monotonic()
        elif measuring:
            done_in_window.append(r)
        inflight.append(submit(k))
        k += 1
    st = srv.stats()
    win = time.monotonic() - t_win
    collect(inflight)
    lat = np.array([r["t_done"] - r["t_submit"] for r in done_in_window]) * 1e3
    peak = {"mode": "closed loop, 512 requests in flight", "seconds": win, "requests": len(done_in_window),
            "steps_per_s": st["track_steps"] / win, "requests_per_s": len(done_in_window) / win,
            "request_ms_p50": float(np.percentile(lat, 50)), "request_ms_p99": float(np.percentile(lat, 99)),
            "batch_ms_p50": st["batch_ms_p50"], "batch_ms_p99": st["batch_ms_p99"], "iterations": st["iterations"],
            "mean_tracks_per_iteration": st["track_steps"] / max(1, st["iterations"])}
    levels = {}
    for frac in (0.25, 0.5, 0.9):
        rate = frac * peak["requests_per_s"]
        duration = 2.0
        srv.reset_stats()
        arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.5) + 16))
        arr = arr[arr < duration]
        ids = []
        t0 = time.monotonic()
        for k, ta in enumerate(arr):
            d = ta - (time.monotonic() - t0)
            if d > 0:
                time.sleep(d)
            ids.append(submit(k))
        res = collect(ids)
        s = summary(res, min(r["t_submit"] for r in res), srv.stats())
        s["offered_requests_per_s"] = rate
        levels[f"{int(frac * 100)}%"] = s
    cap = srv.capacity
    srv.close()
    ctx.close()
    return {"workload": "event stream: requests log-normal (median 2k tracks, sigma 1.5, clipped [1, 500k]), "
                        "mix of the 4M-track step, 16 GB admission budget, resident until < 1 keV or 1000 steps",
            "capacity_tracks": cap, "event_pool": len(events), "event_size_median": int(np.median(sizes)),
            "event_size_max": int(sizes.max()), "peak": peak, "poisson": levels,
            "form": "precision (hepem_server_config.precision = 1)" if args.form == "mixed" else "FP64 batched"}


# ---- distribution checks of the sampled interaction models ----------------------------
MEC2 = 0.51099890999999997


def kn_cdf(eps, k):
    """CDF of eps = E'/E of Klein-Nishina Compton scattering at k = E / m_e c^2:
    the integral of 1/eps + eps - sin^2(theta), 1 - cos(theta) = (1 - eps) / (k eps),
    over [1 / (1 + 2k), eps], in closed form."""
    import numpy as np

    def F(e):
        le = np.log(e)
        return le + 0.5 * e * e - (2.0 / k) * (le - e) + (1.0 / (k * k)) * (-1.0 / e - 2.0 * le + e)

    e0 = 1.0 / (1.0 + 2.0 * k)
    return (F(np.asarray(eps, dtype=np.float64)) - F(e0)) / (F(1.0) - F(e0))


def kn_equal_count_edges(e_mev, nb):
    """Bin edges in eps with equal Klein-Nishina probability (bisection on kn_cdf)."""
    import numpy as np
    k = e_mev / MEC2
    lo = np.full(nb - 1, 1.0 / (1.0 + 2.0 * k))
    hi = np.ones(nb - 1)
    target = np.arange(1, nb) / nb
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        below = kn_cdf(mid, k) < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return np.concatenate([[1.0 / (1.0 + 2.0 * k)], 0.5 * (lo + hi), [1.0]])


def chi2_pvalue(c2, ndf):
    try:
        from scipy.stats import chi2 as _c2
        return float(_c2.sf(c2, ndf))
    except Exception:
        return None


def chi2_expected(counts, probs):
    """Pearson chi2 of counts against bin probabilities; ndf = bins - 1."""
    import numpy as np
    counts = np.asarray(counts, dtype=np.float64)
    exp = counts.sum() * np.asarray(probs, dtype=np.float64)
    c2 = float(np.sum((counts - exp) ** 2 / exp))
    ndf = len(counts) - 1
    return {"chi2": c2, "ndf": ndf, "p_value": chi2_pvalue(c2, ndf)}


def chi2_two_sample(a, b):
    """Two-sample chi2 of histograms a, b (any totals) over the bins where
    either has counts; ndf = those bins - 1."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = (a + b) > 0
    a, b = a[m], b[m]
    ra, rb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    c2 = float(np.sum((ra * a - rb * b) ** 2 / (a + b)))
    ndf = int(m.sum()) - 1
    return {"chi2": c2, "ndf": ndf, "p_value": chi2_pvalue(c2, ndf)}


def sample_histograms(torch, ctx, draws, chunk, seed0):
    """Histograms of independent draws of the FP64 and the FP32 model, each
    from its own seeds (seed0 + c for FP64 chunk c, seed0 + 1000 + c for FP32):
    Seltzer-Berger brem at 999 MeV in G4_Pb in 100 bins of ln(k/E) over
    [ln 1e-4, 0], and Klein-Nishina Compton at 1 MeV in G4_lAr in 100 bins of
    eps = E'/E of equal Klein-Nishina probability.  Returns
    {model: {"fp64": counts, "fp32": counts, "probs": expected or None,
    "fallback": FP32 draws redone in FP64, "draws_per_s": {...}}}."""
    import math
    import numpy as np
    out = {}
    for name, model, e_mev, imc in (("sb_999MeV_G4_Pb", "sb", 999.0, 2), ("compton_1MeV_G4_lAr", "compton", 1.0, 1)):
        if model == "compton":
            edges = torch.from_numpy(kn_equal_count_edges(e_mev, 100)).cuda()
        else:
            edges = torch.linspace(math.log(1e-4), 0.0, 101, dtype=torch.float64, device="cuda")
        rec = {"fallback": 0, "draws_per_s": {}}
        for mixed in (False, True):
            h = torch.zeros(100, dtype=torch.float64, device="cuda")
            t_ms = 0.0
            for c in range(draws // chunk):
                t0 = torch.cuda.Event(enable_timing=True)
                t1 = torch.cuda.Event(enable_timing=True)
                t0.record()
                x, fb = ctx.sample_model(model, chunk, e_mev, imc, seed0 + (1000 if mixed else 0) + c, mixed=mixed)
                t1.record()
                torch.cuda.synchronize()
                t_ms += t0.elapsed_time(t1)
                if mixed:
                    rec["fallback"] += int(fb.item())
                y = x / e_mev
                if model == "sb":
                    y = torch.log(y.clamp_min(1e-300))
                idx = torch.bucketize(y, edges[1:-1], right=True)
                inside = (y >= edges[0]) & (y <= edges[-1])
                h += torch.bincount(idx[inside], minlength=100).double()
            rec["fp32" if mixed else "fp64"] = h.cpu().numpy()
            rec["draws_per_s"]["fp32" if mixed else "fp64"] = draws / (t_ms / 1e3)
        rec["probs"] = np.full(100, 0.01) if model == "compton" else None
        out[name] = rec
    return out


def chi2_report(hists, draws):
    """chi2 of independent FP32 and FP64 samples against each other, and of
    Klein-Nishina samples against the analytic spectrum."""
    rep = {}
    for name, r in hists.items():
        d = {"draws_per_arm": draws, "bins": 100, "streams": "independent seeds per arm",
             "fp32_vs_fp64": chi2_two_sample(r["fp32"], r["fp64"]), "fp64_fallback_draws": r["fallback"],
             "draws_per_s": r["draws_per_s"]}
        if r["probs"] is not None:
            d["fp32_vs_analytic"] = chi2_expected(r["fp32"], r["probs"])
            d["fp64_vs_analytic"] = chi2_expected(r["fp64"], r["probs"])
        rep[name] = d
    return rep


def c5_precision(torch, N, args, n_tracks=1 << 24):
    """Precision: the precision form (hepem_step_mixed) on a
    16,777,216-track batch with the mix of the 4M-track step, against the FP64
    batched form on identical uniforms: steps/s of both, the FP64 fallback
    fraction, discrete mismatches (must be 0) and per-quantity max / RMS
    relative errors; the 2^20-track electron lookups from the FP32 tables against
    the FP64 ones; and chi2 of 1e8 Seltzer-Berger brem draws at 999 MeV in G4_Pb
    (just below the 1 GeV switch to the relativistic model) and 1e8
    Klein-Nishina draws at 1 MeV in G4_lAr, FP32 models against FP64 models
    on independent streams, Klein-Nishina also against the analytic spectrum."""
    from g4hepem_gb300 import workload as W
    ctx = N.Context(TABLE)
    n = n_tracks
    st = W.mixed_batch(n, n_couples=3, seed=WORKLOAD_SEED + 1)
    sin = N.state_to_torch(st)
    del st
    u = N.fill_uniforms(sin["id"], NU, SEED)
    outs, ress, cnts, ms = {}, {}, {}, {}
    for form in ("batched", "mixed"):
        sout = N.empty_state_torch(n)
        res = N.alloc_out_torch(n)
        cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
        for _ in range(max(3, args.warmup)):
            ctx.step(sin, sout, u, NU, SEED, res, form=form)
        torch.cuda.synchronize()
        reps = max(3, min(args.steps, 8))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            ctx.step(sin, sout, u, NU, SEED, res, form=form)
        e1.record()
        torch.cuda.synchronize()
        ms[form] = e0.elapsed_time(e1) / reps
        ctx.step(sin, sout, u, NU, SEED, res, counters=cnt, form=form)
        torch.cuda.synchronize()
        outs[form], ress[form], cnts[form] = sout, res, cnt
    a_s, b_s, a_r, b_r = outs["batched"], outs["mixed"], ress["batched"], ress["mixed"]
    charged = sin["type"] != 2
    mism = {f: int((a_r[f] != b_r[f]).sum()) for f in ("winner", "n_sec", "flags")}
    mism.update({f: int((a_s[f] != b_s[f]).sum()) for f in ("rng_cursor", "gauss_valid")})
    mism["stopped"] = int(((a_s["ekin"] == 0) != (b_s["ekin"] == 0)).sum())

    def rel(x, y, mask=None):
        d = (x - y).abs() / y.abs().clamp_min(1e-300)
        d = torch.where(y == 0, (x - y).abs(), d)
        if mask is not None:
            d = d[mask]
        if d.numel() == 0:
            return None
        return {"max": float(d.max()), "rms": float(d.pow(2).mean().sqrt())}

    ns = a_r["n_sec"].long()
    valid = torch.stack([ns > 0, ns > 1], dim=1).reshape(-1)
    errs = {"ekin": rel(b_s["ekin"], a_s["ekin"]), "edep": rel(b_r["edep"], a_r["edep"]),
            "gstep": rel(b_r["gstep"], a_r["gstep"]), "pstep": rel(b_r["pstep"], a_r["pstep"]),
            "secondary_ekin": rel(b_r["sec_ekin"], a_r["sec_ekin"], valid),
            "msc_tlimit_min": rel(b_s["msc_tlimit_min"], a_s["msc_tlimit_min"], charged),
            "dir_abs_max": float(max((b_s[k] - a_s[k]).abs().max() for k in ("dir_x", "dir_y", "dir_z")))}
    del outs, ress, a_s, b_s, a_r, b_r
    torch.cuda.empty_cache()
    # the 2^20-track electron lookups, FP32 tables against FP64
    e_np, i_np = W.electron_lookup_batch(1 << 20, seed=11)
    ekin = torch.from_numpy(e_np).cuda()
    imc = torch.from_numpy(i_np).cuda()
    l64 = ctx.electron_lookup(ekin, imc)
    l32 = ctx.electron_lookup(ekin, imc, mixed=True)
    torch.cuda.synchronize()
    lookups = {k: rel(l32[k], l64[k]) for k in l64}
    # chi2 of the sampled energies: 1e8 draws per model and precision, each
    # arm from its own seeds; Klein-Nishina also against its analytic spectrum
    chi = chi2_report(sample_histograms(torch, ctx, 10 ** 8, 10 ** 7, SEED + 100), 10 ** 8)
    ctx.close()
    c = cnts["mixed"].cpu().numpy()
    return {"workload": f"{n} mixed tracks (mix of the 4M-track step), 64 Philox uniforms/track, identical streams",
            "mixed": {"value": n / (ms["mixed"] / 1e3), "unit": UNIT, "ms_per_step": ms["mixed"],
                      "entry_point": "hepem_step_mixed"},
            "fp64_batched": {"value": n / (ms["batched"] / 1e3), "unit": UNIT, "ms_per_step": ms["batched"]},
            "speedup_vs_fp64_batched": ms["batched"] / ms["mixed"],
            "fp64_fallback_tracks": int(c[12]), "fp64_fallback_fraction_of_charged": int(c[12]) / int(charged.sum()),
            "discrete_mismatches": mism, "rel_errors": errs, "lookup_rel_errors_c1": lookups, "chi2": chi}


class CpuPort:
    """The oracle's CPU port (the reference algorithm, bit-exact with the
    reference build) stepping the first `n_sample` tracks of a workload on
    `threads` host threads.  Set-up (tables, uniforms, output arrays) happens
    once; `step()` times one pass of the port's step alone."""

    def __init__(self, state, threads, n_sample):
        from oracle import oracle as O
        O.build_port()
        self.port = O.PortLib().load(TABLE)
        sub = {k: np.ascontiguousarray(v[:n_sample]) for k, v in state.items()}
        u = self.port.fill_uniforms(sub["id"], NU, SEED)
        self.run = self.port.step_mt_fn(sub, O.copy_state(sub), O.alloc_out(n_sample), u, NU, SEED, threads)
        self.n = n_sample
        self.threads = threads

    def step(self) -> float:
        t0 = time.perf_counter()
        self.run()
        return time.perf_counter() - t0

    def close(self):
        self.run = None
        self.port.close()


def run_reference(args, ws, rank):
    """CPU reference arm: the oracle port on all host threads (rank 0 only)."""
    if rank != 0:
        return
    from g4hepem_gb300 import workload as W
    threads = os.cpu_count() or 1
    n_sample = args.n
    port = CpuPort(W.mixed_batch(n_sample, seed=WORKLOAD_SEED), threads, n_sample)
    times = []
    for i in range(args.warmup + args.steps):
        dt = port.step()
        if i >= args.warmup:
            times.append(dt)
    port.close()
    tot_time = sum(times)
    value = n_sample * len(times) / tot_time
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_time / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n_sample} tracks of the workload per step, {threads} host threads; "
                                       "the CPU port is bit-exact with the reference build (tests/golden)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    # tracks per step and rank (--tracks: the same, for launches under torchrun,
    # whose own parser would take --n for an abbreviation of its options)
    ap.add_argument("--n", "--tracks", dest="n", type=int, default=N_TRACKS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c3", action="store_true")
    ap.add_argument("--no-c4", action="store_true")
    ap.add_argument("--no-c5", action="store_true")
    ap.add_argument("--no-f", action="store_true", help="skip the stacking and Woodcock rows")
    ap.add_argument("--form", default="mixed", choices=["mixed", "batched"],
                    help="form timed as the headline value (the other FP64 forms are reported beside it)")
    args = ap.parse_args()
    ws, rank, lrank = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(lrank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from g4hepem_gb300 import build as B
    B.build()
    from g4hepem_gb300 import native as N
    from g4hepem_gb300 import workload as W

    n = args.n
    ctx = N.Context(TABLE)
    st_np = W.mixed_batch(n, seed=WORKLOAD_SEED, id0=shard_id0(rank, n))
    sin = N.state_to_torch(st_np)
    sout = N.empty_state_torch(n)
    res = N.alloc_out_torch(n)
    u = N.fill_uniforms(sin["id"], NU, SEED)
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # warm-up (and one counted step for the algorithmic byte count)
    for i in range(max(args.warmup, 3)):
        ctx.step(sin, sout, u, NU, SEED, res, counters=cnt if i == 0 else None, form="batched")
    torch.cuda.synchronize()
    c = cnt.cpu().numpy()
    uniforms_consumed, secondaries = int(c[1]), int(c[3])

    def timed(form, steps):
        """K steps of one form between barriers; max over ranks; ms per step."""
        for _ in range(args.warmup):
            ctx.step(sin, sout, u, NU, SEED, res, form=form)
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            ctx.step(sin, sout, u, NU, SEED, res, form=form)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        t = max_over_ranks(torch, ev0.elapsed_time(ev1), ws)
        return t / steps

    # the plain form (one thread per track) is the denominator of the target;
    # the FP64 batched form and the precision form are timed beside it
    ms_plain = timed("plain", max(3, args.steps // 3))
    other = "batched" if args.form == "mixed" else "mixed"
    ms_other = timed(other, args.steps)
    clocks = Clocks(lrank)
    clocks.start()
    time.sleep(0.3)
    ms_step = timed(args.form, args.steps)
    clk = clocks.stop()
    value = whole_job_rate(ws, n, 1, ms_step / 1e3)
    fcnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    ctx.step(sin, sout, u, NU, SEED, res, counters=fcnt, form="mixed")
    torch.cuda.synchronize()
    fallback = int(fcnt[12].item())

    # e2e through the host-buffer entry point
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()  # noqa: E731
        h_in = {k: pin(v) for k, v in st_np.items()}
        h_out = {k: torch.empty_like(v).pin_memory() for k, v in h_in.items()}
        h_res = {k: torch.from_numpy(v).pin_memory() for k, v in N.alloc_out_numpy(n).items()}
        ctx_steps = max(3, min(args.steps, 10))
        N.lib()
        import ctypes as C
        sin_h, sout_h, sres_h = N.make_state_struct(h_in), N.make_state_struct(h_out), N.make_out_struct(h_res)
        hcnt = N.StepCounters()

        host_fn = N.lib().hepem_step_host_mixed if args.form == "mixed" else N.lib().hepem_step_host

        def host_step():
            # n_uniform = 0: every uniform is drawn on the device from the
            # counter-based stream (seed, track id, k) that fill_uniforms writes
            # into the buffer of the device-resident runs: the same values, so the
            # same results, without moving 8 * NU bytes per track over the link
            N.check(host_fn(ctx.h, n, C.byref(sin_h), C.byref(sout_h), None, 0, SEED, C.byref(sres_h),
                            C.byref(hcnt), stream.cuda_stream))
        for _ in range(3):
            host_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(ctx_steps):
            host_step()
        t_e2e = max_over_ranks(torch, time.perf_counter() - t0, ws)
        h2d = sum(v.numel() * v.element_size() for v in h_in.values())
        d2h = sum(h_out[k].numel() * h_out[k].element_size() for k in N.STATE_OUT_FIELDS)
        d2h += sum(v.numel() * v.element_size() for v in h_res.values())
        link = host_link_gbs(torch)
        moved = (h2d + d2h) / (t_e2e / ctx_steps) / 1e9
        e2e = {"value": whole_job_rate(ws, n, ctx_steps, t_e2e), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": ctx_steps, "ms_per_step": 1e3 * t_e2e / ctx_steps,
               "host_link": {"achieved_gbs": moved, "measured_gbs": link, "frac": moved / link,
                             "note": "e2e is bound by the host<->device copies: measured = concurrent pinned "
                                     "H2D + D2H copies of 2 GiB each (torch)"},
               "entry_point": ("hepem_step_host_mixed" if args.form == "mixed" else "hepem_step_host")
               + " (pinned host buffers)",
               "uniforms": "n_uniform = 0: drawn on the device from the same (seed, id, k) stream as the "
                           "buffer of the device-resident runs (identical results), not copied"}
        if args.form == "mixed":
            # the bit-exact FP64 form end to end as well (reference precision)
            host_fn = N.lib().hepem_step_host
            host_step()
            barrier()
            t0 = time.perf_counter()
            for _ in range(ctx_steps):
                host_step()
            t_64 = max_over_ranks(torch, time.perf_counter() - t0, ws)
            e2e["fp64_batched"] = {"value": whole_job_rate(ws, n, ctx_steps, t_64), "unit": UNIT,
                                   "ms_per_step": 1e3 * t_64 / ctx_steps,
                                   "entry_point": "hepem_step_host (pinned host buffers)"}

    if rank != 0:
        return
    hbm, hbm_src = peaks()
    c1 = c1_lookups(torch, N, ctx, stream, args, hbm)
    c3 = None if args.no_c3 else c3_batching(torch, N, args)
    c4 = None if args.no_c4 else c4_serving(torch, N, args)
    c5 = None if args.no_c5 else c5_precision(torch, N, args)
    # the rows after the step, on the precision-form step's results
    ctx.step(sin, sout, u, NU, SEED, res, form="mixed")
    torch.cuda.synchronize()
    rows_f = None if args.no_f else f_rows(torch, N, ctx, sout, res, hbm)
    # per-stage device times of one more step of each batched form: CUDA events
    # recorded on the launching stream around every stage (hepem_profile_stages)
    import ctypes as C

    def stage_times(form):
        N.check(N.lib().hepem_profile_stages(ctx.h, 1))
        ctx.step(sin, sout, u, NU, SEED, res, form=form)
        ms_c, nm_c, cnt_c = (C.c_float * 16)(), (C.c_char_p * 16)(), C.c_int32()
        N.check(N.lib().hepem_stage_times(ctx.h, ms_c, nm_c, 16, C.byref(cnt_c)))
        N.check(N.lib().hepem_profile_stages(ctx.h, 0))
        return {nm_c[i].decode(): float(ms_c[i]) for i in range(cnt_c.value)}

    stages = {"mixed": stage_times("mixed"), "batched": stage_times("batched")}
    head = stages[args.form]
    dom = max(head, key=head.get)
    ms_dom = head[dom]
    # dominant kernel: e+- stage A (with its FP64 fallback in the precision
    # form).  Algorithmic bytes per e+- track: input state 128 B, output state
    # 102 B, step results 51 B, queue entry 4 B, and 8 B per uniform the track
    # consumed in the step (cursor sum, a slight overestimate for stage A alone).
    charged = st_np["type"] != 2
    n_ch = int(charged.sum())
    cur = sout["rng_cursor"].cpu().numpy()
    alg = n_ch * (128 + 102 + 51 + 4) + 8 * int(cur[charged].sum())
    achieved = alg / (ms_dom / 1e3) / 1e9
    prof = profile_summary("stage_a_charged_mixed.json" if args.form == "mixed" else "stage_a_charged.json")
    traffic = prof["dram_bytes_per_track"] * n_ch if prof else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_src == "measured" else "fallback",
            "algorithmic_bytes_per_launch": alg, "ms_per_launch": ms_dom,
            "note": ("HBM is not the limit of this kernel: the precision form's stage A is bound by the latency "
                     "of dependent table and state gathers; traffic is the ncu DRAM bytes per e+- track x the e+- "
                     "tracks of the step" if args.form == "mixed" else
                     "HBM is not the limit of this kernel: the FP64 pipe is (roofline_fp64)")}
    fp64 = {"bound": "fp64", "kernel": dom, "unit": "TFLOP/s", "peak": None,
            "peak_source": "measured here: cuBLAS DGEMM 4096^3 (MEASURED_PEAKS.json has no FP64 figure)"}
    fp32 = {"bound": "fp32", "kernel": dom, "unit": "TFLOP/s", "peak": None,
            "peak_source": "measured here: cuBLAS SGEMM 8192^3, TF32 off (MEASURED_PEAKS.json has no FP32 figure)"}
    try:
        fp64["peak"] = fp64_peak_tflops(torch)
        fp32["peak"] = fp32_peak_tflops(torch)
    except Exception as ex:  # pragma: no cover
        fp64["error"] = str(ex)
    for rf, key in ((fp64, "dflop_per_track"), (fp32, "sflop_per_track")):
        if prof and rf["peak"] and key in prof:
            flops = prof[key] * n_ch
            rf["achieved"] = flops / (ms_dom / 1e3) / 1e12
            rf["frac"] = rf["achieved"] / rf["peak"]
            rf["flops_per_launch"] = flops
            rf[key] = prof[key]
    cpu = None
    if not args.no_cpu:
        # every track of the step, passes repeated for about 10 s of CPU work
        threads = os.cpu_count() or 1
        port = CpuPort(st_np, threads, n)
        port.step()  # warm
        times = []
        while len(times) < 2 or (sum(times) < 10.0 and len(times) < 200):
            times.append(port.step())
        port.close()
        dt = sum(times)
        cpu = {"value": n * len(times) / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"all {n} tracks of the step, {len(times)} passes ({dt:.1f} s of stepping), "
                         f"{threads} host threads"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.form == "mixed" else "f64", "data": "synthetic", "config": CONFIG, "e2e": e2e,
            "gpu_launches": (LAUNCHES_PER_STEP_MIXED if args.form == "mixed" else LAUNCHES_PER_STEP) * args.steps,
            "form": ("precision form (hepem_step_mixed): discrete outcomes of the FP64 path, continuous within "
                     "1e-5" if args.form == "mixed" else
                     "batched FP64 (hepem_step_batched): bit-identical to the plain FP64 path"),
            "fp64_fallback_per_step": fallback,
            "plain_fp64": {"value": whole_job_rate(ws, n, 1, ms_plain / 1e3), "unit": UNIT, "ms_per_step": ms_plain,
                           "entry_point": "hepem_step"},
            ("batched_fp64" if other == "batched" else "mixed"): {
                "value": whole_job_rate(ws, n, 1, ms_other / 1e3), "unit": UNIT, "ms_per_step": ms_other,
                "entry_point": "hepem_step_batched" if other == "batched" else "hepem_step_mixed"},
            "vs_plain_fp64": ms_plain / ms_step, "roofline": roof, "roofline_fp64": fp64, "roofline_fp32": fp32,
            "stage_ms": stages, "c1_lookup": c1, "c3_batching": c3, "c4_serving": c4, "c5_precision": c5,
            "f_rows": rows_f,
            "cpu_baseline": cpu, "clocks": clk,
            "counters": {"uniforms_per_step": uniforms_consumed, "secondaries_per_step": secondaries,
                         "interactions": [int(x) for x in c[4:12]]}}
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
