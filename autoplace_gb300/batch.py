"""Batches of uneven placement instances (floorplan variants, seeds, blocks) in one CUDA graph.

The reference places one design per process, with a host poll every 16 passes (src/gpu_loop.py:58-70). Here a batch
of N independent instances -- each with its own netlist, grid and field mode -- runs as:
  1. the start positions of every instance uploaded (Placer.load);
  2. ONE graph with every instance's whole placement (gp103_batch_add_run): per instance an IF node with the level's
     set-up (gp103_begin: the step-length probes and the start's state), a conditional WHILE node looping 4 passes
     of the wirelength-only start until that instance's start phase ends, an IF node with the hand-over to the
     density phase (the first density weight from the tension unit, the density phase's state), and a WHILE node
     looping 8 passes (the first refreshing the scatter's spatial order) until the instance's control stops it;
  3. the placements (Placer.start_over, Placer.end).
The instances are separate branches of the graph, so the GPU runs them side by side; no host step happens between
the set-up and the stop. Results are those of Placer.run for each instance, bit for bit (the same kernels in
the same order; passes after a stop change nothing). The device time at which each instance's density loop ends is
recorded, which gives each instance's time to the stop from the batch's start.
"""
import ctypes
import time

import numpy as np
import torch

from . import native
from .engine import Placer

START_PASSES, DENSITY_PASSES = 4, 8


class _Graph(object):
    def __init__(self, placers, stream, dev):
        n = len(placers)
        self.loops = torch.zeros((n, 2), dtype=torch.int32, device=dev)       # bodies of the start, density loops
        self.stop_ns = torch.zeros((n, 2), dtype=torch.int64, device=dev)
        self.t0 = torch.zeros(1, dtype=torch.int64, device=dev)
        h = ctypes.c_void_p()
        native.call("gp103_batch_create", ctypes.byref(h))
        self.h = h
        for k, pl in enumerate(placers):
            o = pl.p.opts
            args = pl.begin_args(pl.start_gamma)
            native.call("gp103_batch_add_run", h, pl._ref, ctypes.byref(args), START_PASSES, DENSITY_PASSES,
                        int(o.inner_iter) // START_PASSES + 2, int(o.inner_iter) // DENSITY_PASSES + 2,
                        float(o.density_weight), float(pl.p.total_pins), float(pl.start_gamma), pl._p(pl.tmp[0]),
                        pl._p(pl.tmp[1]), pl._p(pl.scal), ctypes.c_void_p(self.loops.data_ptr() + 8 * k),
                        ctypes.c_void_p(self.stop_ns.data_ptr() + 16 * k), stream.cuda_stream)

    def launch(self, stream):
        with torch.cuda.stream(stream):
            self.loops.zero_()
        native.call("gp103_batch_launch", self.h, ctypes.c_void_p(self.t0.data_ptr()), stream.cuda_stream)

    def __del__(self):
        try:
            native.lib().gp103_batch_destroy(self.h)
        except Exception:
            pass


class Batch(object):
    """N instances (Problems) placed together. fields: one field mode per instance (or one for all); tuned: per-
    instance settings from tune.py (field mode and the WA lane groups), applied before the graph is captured."""

    def __init__(self, problems, fields="f16x3", device="cuda", tuned=None):
        self.dev = torch.device(device)
        self.stream = torch.cuda.Stream(self.dev)
        n = len(problems)
        fields = fields if isinstance(fields, (list, tuple)) else [fields] * n
        if tuned:
            fields = [t.get("field", f) for t, f in zip(tuned, fields)]
        self.placers = [Placer(p, field=f, device=self.dev, use_graphs=False, stream=self.stream)
                        for p, f in zip(problems, fields)]
        if tuned:
            from . import tune
            for pl, t in zip(self.placers, tuned):
                tune.apply_wa(pl, t.get("wa", "default"))
        self.stream.synchronize()
        self.graph = _Graph(self.placers, self.stream, self.dev)

    def run(self, pos0s):
        """Place every instance from its start positions. -> (list of Placer.run result dicts, per-instance seconds
        from the batch's start to the end of its density loop, device-timed, and the batch's wall seconds)."""
        torch.cuda.synchronize(self.dev)
        t0 = time.time()
        for pl, p0 in zip(self.placers, pos0s):
            pl.load(p0)
        self.graph.launch(self.stream)
        self.stream.synchronize()
        results = []
        for pl in self.placers:
            ctx = pl.context(t0)
            out = pl.start_over(ctx, pl.T.cpu().numpy())         # the result when the start phase stopped the run
            results.append(out if out is not None else pl.end(ctx))
        wall = time.time() - t0
        stop = self.graph.stop_ns[:, 1].cpu().numpy().astype(np.int64)
        per = (stop - int(self.graph.t0.cpu()[0])) / 1e9
        return results, per, wall
