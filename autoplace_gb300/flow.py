"""Global placement of one design: one level, or two (the clusters first, then the cells), on the device.

Mirrors global_placement_main (src/run_placement.py:79-122):
  - cluster_ratio <= 1: one level of the cells (engine.Placer.run);
  - cluster_ratio > 1 (two levels):
      1. the clusters and their problem (cluster.coarse_problem: star matching, pins and sizes on the device);
      2. one level of the clusters, with no settle and no minimum iteration count, stopped ("handover") once its
         smoothing is down to the one the cells start with (10 x the cells' base gamma);
      3. the cells spread over their clusters' squares (cluster.expand) and clamped into the region;
      4. the density weight carried over in tension units: weight = lam of the clusters x tension unit of the cells
         / tension unit of the clusters (the same share of the wire tension on both levels); the smoothing in units
         of the bin (wa_rule accuracy) or from the cells' overflow (wa_rule overflow); the scheduler's iteration
         count and the cells' HPWL (ParamScheduler.resume);
      5. one level of the cells from there, counted on from the clusters' last iteration, with no wirelength-only
         start.
"""
import time

import torch

from . import cluster
from .engine import Placer, side_stream


def _gamma(base_gamma, overflow):
    """ParamScheduler.gamma (src/param_scheduler.py:50-51): the smoothing of the overflow rule."""
    return base_gamma * 10 ** ((overflow - 0.1) * 20 / 9 - 1)


class Flow(object):
    """A design's global placement, reusable: the cells' Placer is set up once and every run() places from a start
    (the clusters, their problem and their Placer are made per run, as the reference makes them per placement).

    field: the cells' field mode; coarse_field: the clusters' (default: the same; a grid the tensor cores cannot tile
    runs in fp32). split: the WA kernels of density passes on a second stream (Placer(split=True)), on both levels. start: None = the reference's start (the clusters from the start positions with the wirelength-
    only start); or a callable start(coarse, cplacer, cpos0, prob) -> (cluster positions [num + F, 2] on the device,
    resume dict or None) that proposes the clusters' positions (and the density weight and smoothing to resume the
    clusters' level with, ParamScheduler.resume) in place of the wirelength-only start."""

    def __init__(self, prob, field="f16x3", coarse_field=None, device="cuda", check_every=16, use_graphs=True,
                 stream=None, host=None, split=True):
        self.prob = prob
        self.dev = torch.device(device)
        self.stream = stream or torch.cuda.Stream(self.dev)
        self.kw = dict(device=self.dev, check_every=check_every, use_graphs=use_graphs, stream=self.stream)
        self.field, self.coarse_field = field, coarse_field or field
        # density passes with the WA kernels on a second stream, beside the density map and the field, on both levels
        # (gp103_pass_split; the same runs bit for bit): at the 1.2M-cell netlist the clusters' level 38.2 -> 35.5 ms,
        # the cells' level 46.3 -> 44.9 ms
        self.split = bool(split)
        self.side = side_stream(self.stream) if self.split else None
        # what every placement's clustering needs of the design (pins on the device, areas, limits, seeded draws);
        # first, so that its seeded draws (on background threads) run beside the cells' Placer's set-up
        self.prep = (cluster.prepare(prob, device=self.dev, stream=self.stream, draw_stream=self.side)
                     if prob.opts.cluster_ratio > 1 else None)
        self.fine = Placer(prob, field=field, host=host, split=self.split, side=self.side, **self.kw)
        self.last_coarse = None
        self.keep_coarse_placer = False             # keep the clusters' Placer of the last run (last_cplacer)
        self.last_cplacer = None

    def run(self, pos0, log=None, start=None, fallback=True):
        """Place from pos0 ([num_nodes, 2], movable cells then fillers). -> dict of statistics as the reference's
        (stop_reason, iters, start_iters, gp_time_s, per_iter_s, grad_calls; with two levels also clusters,
        cluster_time_s, coarse_num_bin, coarse_iters) plus pos (final positions on the device), hpwl and overflow of
        the kept placement as the control measured them, and placer (the cells' Placer: placer.evaluate(pos) gives
        the exact HPWL and overflow). fallback: a placement from a `start` proposal that does not converge is placed
        again from the reference's start (stats["fallback"] = True)."""
        st = self._run(pos0, log, start)
        if start is not None and fallback and st["stop_reason"] != "converged":
            if log:
                log("the proposal's placement stopped (%s): placed again from the plain start" % st["stop_reason"])
            st = self._run(pos0, log, None)
            st["fallback"] = True
        return st

    def _run(self, pos0, log, start):
        prob, fine, stream, dev = self.prob, self.fine, self.stream, self.dev
        o, n = prob.opts, prob.num_mov
        torch.cuda.synchronize(dev)
        t0 = time.time()
        stats, evals, resume, start_iters = {}, 0, None, 0
        marks = [("begin", t0)]                     # wall times at phase ends (each after a host synchronisation)
        if o.cluster_ratio > 1:
            coarse = cluster.coarse_problem(prob, device=dev, stream=stream, prep=self.prep)
            cp = coarse.problem
            stream.synchronize()
            stats = dict(clusters=coarse.num, cluster_time_s=time.time() - t0, coarse_num_bin=cp.force.nbx)
            marks.append(("clustering", time.time()))
            if log:
                log("two levels: %d clusters of %d cells (%.2fs), %d x %d bins"
                    % (coarse.num, n, stats["cluster_time_s"], cp.force.nbx, cp.force.nby))
            start_gamma = 10 * prob.base_gamma                      # the smoothing the cells start with
            cplacer = Placer(cp, field=self.coarse_field, handover_gamma=start_gamma, split=self.split,
                             side=self.side, **self.kw)
            marks.append(("cluster_setup", time.time()))
            with torch.cuda.stream(stream):
                p0 = torch.as_tensor(pos0, dtype=torch.float32).to(dev)
                cpos0 = torch.cat([p0[:coarse.num], p0[n:]])
            cresume = None
            if start is not None:
                t1 = time.time()
                cpos0, cresume = start(coarse, cplacer, cpos0, prob)
                stream.synchronize()
                stats["start_time_s"] = time.time() - t1
            if start is not None:
                marks.append(("proposal", time.time()))
            level = cplacer.run(cpos0, log=log, resume=cresume)
            marks.append(("cluster_level", time.time()))
            cpos = level["pos"]
            pos = cluster.expand(cpos, coarse, prob, o.seed, device=dev, stream=stream)
            with torch.cuda.stream(stream):
                torch.max(torch.min(pos, fine.hi), fine.lo, out=pos)
            # the same share of the wire tension on both levels
            tu_fine, ovf_fine = fine.tension_unit(pos)
            tu_coarse = cplacer.tension_unit(cpos)[0]
            weight = level["lam"] * tu_fine / tu_coarse
            if o.wa_rule == "accuracy":                             # the same smoothing in units of the bin
                gam = level["gam"] / cp.base_gamma * prob.base_gamma
            else:
                gam = _gamma(prob.base_gamma, ovf_fine)
            resume = dict(lam=weight, gam=gam, iter=level["iter"], hpwl=fine.hpwl(pos), first_iter=level["iters"])
            marks.append(("handover", time.time()))
            if log:
                log("clusters placed after %d iterations (stop: %s, hpwl %.4E, overflow %.4f): the cells take over, "
                    "density weight %.4E" % (level["iters"], level["reason"], level["hpwl"], level["overflow"],
                                             weight))
            evals, start_iters = level["evals"], level["start_iters"]
            stats["coarse_iters"] = level["iters"]
            stats["coarse_reason"] = level["reason"]
            pos0 = pos
            self.last_coarse = coarse
            self.last_cplacer = cplacer if self.keep_coarse_placer else None
            del cplacer, cp, cpos                                   # the clusters' buffers are not needed any more
        level = fine.run(pos0, log=log, resume=resume)
        torch.cuda.synchronize(dev)
        marks.append(("cell_level", time.time()))
        stats["phase_s"] = {name: round(t - marks[k][1], 5) for k, (name, t) in enumerate(marks[1:])}
        gp_time, iters = time.time() - t0, level["iters"]
        if log:
            log("GP stop (%s): #iters %d hpwl: %.6E overflow: %.4f GP time: %.4fs per iter: %.6fs (%d gradient calls)"
                % (level["reason"], iters, level["hpwl"], level["overflow"], gp_time, gp_time / max(iters, 1),
                   evals + level["evals"]))
        stats.update(stop_reason=level["reason"], iters=iters, start_iters=start_iters or level["start_iters"],
                     gp_time_s=gp_time, per_iter_s=gp_time / max(iters, 1), grad_calls=evals + level["evals"],
                     pos=level["pos"], hpwl=level["hpwl"], overflow=level["overflow"], placer=fine)
        return stats


def global_placement(prob, pos0, field="f16x3", device="cuda", log=None, check_every=16, use_graphs=True,
                     stream=None, start=None):
    """Place prob from pos0 ([num_nodes, 2], movable cells then fillers): Flow(prob, ...).run(pos0) (see Flow)."""
    return Flow(prob, field=field, device=device, check_every=check_every, use_graphs=use_graphs,
                stream=stream).run(pos0, log=log, start=start)
