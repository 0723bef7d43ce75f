"""NVTX ranges on the GPU paths, recorded by tests/trace/trace_recorder.c: a
batched step, a precision-form step, a split step and the host-buffer step
each open one range named for the entry point with the batch size as
payload, and inside a batched step the stage ranges follow the launch order
(sort, the two stage A kernels, the nine interaction queues in the order of
their streams; the precision form's FP64 fallback last)."""
import pytest

from client_build import run_traced
from conftest import T3

pytestmark = pytest.mark.gpu

STAGES = ["sort", "stage_a_charged", "stage_a_gamma", "ioni_e-", "ioni_e+", "brem_sb", "brem_rb",
          "annihilation_in_flight", "annihilation_at_rest", "conversion", "compton", "photoelectric"]

CODE = """
import numpy as np, torch
from g4hepem_gb300 import native, workload as W
ctx = native.Context({table!r})
n = 4096
st = W.mixed_batch(n, n_couples=3, seed=3)
sin = native.state_to_torch(st)
u = native.fill_uniforms(sin['id'], 32, 9)
for form in ('batched', 'mixed'):
    sout = native.empty_state_torch(n)
    res = native.alloc_out_torch(n)
    ctx.step(sin, sout, u, 32, 9, res, form=form)
gstep, limits = ctx.howfar(sin, u, 32, 9, form='mixed')
sout = native.empty_state_torch(n)
res = native.alloc_out_torch(n)
ctx.perform(sin, sout, gstep, limits, u, 32, 9, res, form='mixed')
torch.cuda.synchronize()
uh = W.philox_uniforms(9, st['id'], 32).reshape(-1)
out = {{k: np.empty_like(v) for k, v in st.items()}}
ctx.step_host(st, out, uh, 32, 9, native.alloc_out_numpy(n), mixed=True)
"""


def tree(ev):
    """[(name, payload, [children])] from the push/pop records."""
    root, stack = [], []
    for e in ev:
        if e[0] == "push":
            node = (e[2], int(e[3]), [])
            (stack[-1][2] if stack else root).append(node)
            stack.append(node)
        else:
            stack.pop()
    assert not stack
    return root


def test_step_ranges(tmp_path):
    ev = run_traced(CODE.format(table=T3), str(tmp_path / "trace.log"))
    assert all(e[1] == "g4hepem_gb300" for e in ev)
    top = [(name, n) for name, n, _ in tree(ev)]
    names = [t[0] for t in top]
    assert names[0] == "hepem_create_from_file", names
    calls = [t for t in top if t[0].startswith("hepem_step") or t[0] in ("hepem_howfar", "hepem_perform")]
    assert [c[0] for c in calls] == ["hepem_step_batched", "hepem_step_mixed", "hepem_howfar", "hepem_perform",
                                     "hepem_step_host_mixed"], calls
    assert all(c[1] == 4096 for c in calls)
    nodes = {name: kids for name, _, kids in tree(ev)}

    def launch_order(kids, expected, fallback):
        names = [k[0] for k in kids]
        # the sort, the two stage A kernels, then the queues (in the order of
        # their streams: the queues overlap on side streams), the FP64
        # fallback of the precision form last
        assert names[:3] == expected[:3], names
        assert sorted(names[3:len(expected)]) == sorted(expected[3:]), names
        assert names[len(expected):] == (["fp64_fallback"] if fallback else []), names

    launch_order(nodes["hepem_step_batched"], STAGES, False)
    launch_order(nodes["hepem_step_mixed"], STAGES, True)
    assert [k[0] for k in nodes["hepem_howfar"]] == STAGES[:3] + ["fp64_fallback"]
    # Perform: the sort, its own stage A kernels (the Perform phase), the queues
    launch_order(nodes["hepem_perform"], STAGES, True)
    assert all(k[1] == 4096 for k in nodes["hepem_step_mixed"])
    # the host-buffer step: one batched step (a chunk of 4096 tracks) inside
    launch_order(nodes["hepem_step_host_mixed"], STAGES, True)
