"""Steps of one form over a synthetic batch, for profilers (ncu) and quick
timings: the bench's workload (mixed e-/e+/gamma tracks, 1 MeV - 10 GeV,
three couples) at a size of choice, a few warm-up steps, then the steps to
capture.

    python -m g4hepem_gb300.profile_step --n 1048576 --form mixed --steps 2

prints one JSON line with the CUDA-event time per step of the captured steps.
"""
from __future__ import annotations

import argparse
import json
import os


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 20, help="tracks per step")
    ap.add_argument("--form", default="mixed", choices=["plain", "batched", "mixed"])
    ap.add_argument("--steps", type=int, default=2, help="steps after the warm-up")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--uniforms", type=int, default=64, help="uniforms per track (0: drawn by the library)")
    ap.add_argument("--seed", type=int, default=7, help="workload seed")
    args = ap.parse_args(argv)

    import torch

    from g4hepem_gb300 import build as B
    B.build()
    from g4hepem_gb300 import native as N
    from g4hepem_gb300 import workload as W

    torch.cuda.set_device(0)
    table = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "three_couples_0.7mm.json")
    ctx = N.Context(table)
    n, nu = args.n, args.uniforms
    sin = N.state_to_torch(W.mixed_batch(n, seed=args.seed))
    sout = N.empty_state_torch(n)
    res = N.alloc_out_torch(n)
    u = N.fill_uniforms(sin["id"], nu, 20261203) if nu else None
    for _ in range(args.warmup):
        ctx.step(sin, sout, u, nu, 20261203, res, form=args.form)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        ctx.step(sin, sout, u, nu, 20261203, res, form=args.form)
    e1.record(s)
    torch.cuda.synchronize()
    print(json.dumps({"form": args.form, "tracks": n, "uniforms_per_track": nu, "steps": args.steps,
                      "ms_per_step": e0.elapsed_time(e1) / max(args.steps, 1)}))


if __name__ == "__main__":
    main()
