"""A fixed profiling case: place one synthetic netlist, then run extra density passes (from the placed state)
inside an NVTX range "gp103_profile", so that a profiler can be limited to them with
--nvtx --nvtx-include "gp103_profile/".

    python -m autoplace_gb300.profile_case --config c2 --passes 8 [--field f16x3]

--flow: the range holds one whole placement of the preset's flow instead (two levels at cluster ratio > 1:
clustering, the clusters' level, the hand-over, the cells' level), after one untimed placement that captures the
CUDA graphs.
"""
import argparse
import time

import torch

from . import native, problem, synth
from .engine import Placer


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--field", default="f16x3")
    ap.add_argument("--passes", type=int, default=8)
    ap.add_argument("--flow", action="store_true")
    a = ap.parse_args(argv)
    nl, o = synth.preset(a.config)
    prob = problem.Problem(nl, problem.options(**o))
    if a.flow:
        from .flow import Flow
        f = Flow(prob, field=a.field)
        pos0 = torch.as_tensor(synth.init_positions(nl, prob.num_nodes)).cuda()
        f.run(pos0)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("gp103_profile")
        st = f.run(pos0)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        print("profiled one placement: %s after %d iterations, %.4f s, phases %s"
              % (st["stop_reason"], st["iters"], st["gp_time_s"], st["phase_s"]))
        return
    pl = Placer(prob, field=a.field)
    pos0 = synth.init_positions(nl, prob.num_nodes)
    t = time.time()
    r = pl.run(pos0)
    print("placed: %s after %d iterations, %.3f s" % (r["reason"], r["iters"], time.time() - t))
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("gp103_profile")
    pl._passes(native.PHASE_DENSITY, a.passes)
    pl.sync()
    torch.cuda.nvtx.range_pop()
    print("profiled %d density passes" % a.passes)


if __name__ == "__main__":
    main()
