"""Batches of uneven placement instances (floorplan variants, seeds, blocks) in one CUDA graph per phase.

The reference places one design per process, with a host poll every 16 passes (src/gpu_loop.py:58-70). Here a batch
of N independent instances -- each with its own netlist, grid and field mode -- runs as:
  1. the host part of every instance (Placer.begin: the step-length probes);
  2. ONE graph for the wirelength-only starts: a conditional WHILE node per instance (gp103_batch_add), looping
     4 passes at a time until that instance's start phase ends;
  3. the first density weight of every instance (Placer.start_end: its tension unit);
  4. ONE graph for the density phases: a WHILE node per instance looping 8 passes (the first refreshing the scatter's
     spatial order) until its control stops it;
  5. the placements (Placer.end).
The instances are separate branches of each graph, so the GPU runs them side by side; no host poll happens inside a
phase. Results are those of Placer.run for each instance, bit for bit (the same kernels in the same order; passes
after a stop change nothing). The device time at which each instance's loop ends is recorded, which gives each
instance's time to the stop from the batch's start.
"""
import ctypes
import time

import numpy as np
import torch

from . import native
from .engine import Placer, SK

START_PASSES, DENSITY_PASSES = 4, 8


class _Graph(object):
    def __init__(self, placers, phase, passes, sort_first, stream, dev):
        n = len(placers)
        self.loops = torch.zeros(n, dtype=torch.int32, device=dev)
        self.stop_ns = torch.zeros(n, dtype=torch.int64, device=dev)
        self.t0 = torch.zeros(1, dtype=torch.int64, device=dev)
        h = ctypes.c_void_p()
        native.call("gp103_batch_create", ctypes.byref(h))
        self.h = h
        for k, pl in enumerate(placers):
            o = pl.p.opts
            max_loops = int(o.inner_iter) // passes + 2
            native.call("gp103_batch_add", h, pl._ref, phase, passes, int(sort_first), max_loops,
                        ctypes.c_void_p(self.loops.data_ptr() + 4 * k),
                        ctypes.c_void_p(self.stop_ns.data_ptr() + 8 * k), stream.cuda_stream)

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
    instance settings from tune.py (field mode and the WA lane groups), applied before the graphs are captured."""

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
        self.start_graph = _Graph(self.placers, native.PHASE_START, START_PASSES, False, self.stream, self.dev)
        self.density_graph = _Graph(self.placers, native.PHASE_DENSITY, DENSITY_PASSES, True, self.stream, self.dev)

    def run(self, pos0s):
        """Place every instance from its start positions. -> (list of Placer.run result dicts, per-instance seconds
        from the batch's start to the end of its density loop, device-timed, and the batch's wall seconds)."""
        torch.cuda.synchronize(self.dev)
        t0 = time.time()
        ctxs = [pl.begin(p0) for pl, p0 in zip(self.placers, pos0s)]
        self.start_graph.launch(self.stream)
        self.stream.synchronize()
        results = [None] * len(self.placers)
        for k, (pl, ctx) in enumerate(zip(self.placers, ctxs)):
            results[k] = pl.start_end(ctx)                 # None, or the result when the start phase stopped
        with torch.cuda.stream(self.stream):
            for k, pl in enumerate(self.placers):          # a finished instance's density loop ends at once
                if results[k] is not None:
                    pl.S[SK["stop"]] = results[k].get("stop_code", 4)
        self.density_graph.launch(self.stream)
        self.stream.synchronize()
        for k, (pl, ctx) in enumerate(zip(self.placers, ctxs)):
            if results[k] is None:
                results[k] = pl.end(ctx)
        wall = time.time() - t0
        start_t0 = int(self.start_graph.t0.cpu()[0])
        stop = self.density_graph.stop_ns.cpu().numpy().astype(np.int64)
        per = (stop - start_t0) / 1e9
        return results, per, wall
