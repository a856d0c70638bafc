"""Benchmark: time to overflow 0.07 of a global placement of the 1.2M-cell synthetic netlist on a GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config c2] [--field f16x3]
                    [--start auto|learned|plain]

Workload (config "c2"): 1,200,000 cells, 1,250,000 nets (5.2M pins, degree mix 2/3/4-10/11-100), 40 macros over 20 %
of the region, target density 0.8, force grid 1024 x 1024, overflow grid 512 x 512, two levels (cluster ratio 5, the
reference's default: the clusters first, then the cells); seeded synthetic data (the ISPD suites are not available).
One step = one whole placement from the seeded start to the stop (clustering, the clusters' level, expansion, the
cells' level until overflow < 0.07 + the settle iterations), inputs resident in HBM. The working set (pins, nodes,
maps, field planes) is larger than the 129 MB L2, so no flush is needed between steps.

Reported on one JSON line (rank 0): value = seconds per placement with the product's configuration (lower is better:
the tensor-core field, and the learned start when a trained model is present), the plain method on the same GPU
beside it (the reference's start and a float32 field), e2e = the same placement through the public API from the
netlist's host arrays (upload, the problem's arrays built on the device, run, download of the placement), the
roofline of the dominant kernel (CUDA events on its stream), a CPU baseline (the oracle's restatement of the
reference's CPU iteration on the host cores, timed on a bounded sample of iterations), SM clocks during the timed
region, and the number of libgp103 kernels launched.

--impl reference: the reference's CPU path (its --gpu -1 PyTorch operators) restated by the oracle on every host core
(float32 operators, FFT field), one whole placement of the same netlist and flow to its own stop, timed in full: its
own iterations, exact HPWL and overflow; the K steps of the line are K consecutive shares of that one placement.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-overflow 0.07 (s) at 1.2M cells, learned+TC vs plain, HPWL within 1%"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="c2")
    p.add_argument("--field", default="f16x3", choices=["f16x3", "bf16x6", "bf16x3", "tf32x3", "fp32"])
    p.add_argument("--start", default="auto", choices=["auto", "learned", "plain"],
                   help="the clusters' start: the learned proposal (auto: when a trained model is present) or the "
                        "reference's wirelength-only start")
    p.add_argument("--plain-field", default="fp32", help="field mode of the plain method beside the measurement")
    p.add_argument("--plain-steps", type=int, default=2, help="timed placements of the plain method")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--cpu-iters", type=int, default=12, help="density-phase iterations of the CPU sample")
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-pdl", action="store_true", help="plain stream order instead of programmatic dependent launch")
    p.add_argument("--split", action="store_true", help="the WA kernels on a second stream, beside the density map")
    p.add_argument("--instances", type=int, default=64, help="--config c3: instances per batch")
    return p.parse_args()


# ------------------------------------------------------------------------------------------------ ranks
def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x, world):
    """Max over ranks of a float (the slowest replica decides the step time)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, world):
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------------------------------------ clocks
class Clocks(object):
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.path = index, None, None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------------ workload
def workload(cfg, seed):
    from autoplace_gb300 import problem, synth
    nl, o = synth.preset(cfg, seed=seed)
    prob = problem.Problem(nl, problem.options(**o))
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=seed)
    return prob, pos0


def config_dict(prob, args, world, start="plain"):
    nl = prob.nl
    levels = 2 if prob.opts.cluster_ratio > 1 else 1
    return {"workload": "synthetic %s: %d cells, %d nets, %d pins, %d macros, %d fillers; force grid %d, overflow grid "
                        "%d; %d level(s)" % (args.config, nl.num_mov, nl.num_nets, nl.num_pins, len(nl.macros),
                                             prob.num_nodes - prob.num_mov, prob.force_bin, prob.num_bin, levels),
            "cells": nl.num_mov, "nets": nl.num_nets, "pins": nl.num_pins, "nodes": prob.num_nodes,
            "force_grid": prob.force_bin, "overflow_grid": prob.num_bin, "target_density": prob.target,
            "cluster_ratio": prob.opts.cluster_ratio, "levels": levels, "field": args.field,
            "start": start, "streams": 2 if args.split else 1,
            "l2": "working set > 129 MB L2 (no flush)", "parallelism": "replicas x%d" % world}


# ------------------------------------------------------------------------------------------------ CPU baseline
def cpu_sample(prob, pos0, iters):
    """Time `iters` density-phase iterations of the oracle's CPU iteration on every host core (float32 WA, density map,
    overflow grid, field by FFT of the mirrored map, gather; Nesterov step; control), after two untimed warm-up
    iterations. -> (seconds per iteration, threads)."""
    import numpy as np
    from oracle import gp_oracle as O
    threads = os.cpu_count() or 1
    lvl = O.CpuLevel(prob, dtype=np.float32, field="fft", threads=threads)
    gr = prob.force
    v = np.clip(np.asarray(pos0, np.float64), gr.pos_lo, gr.pos_hi)
    gam, lam = 10 * prob.base_gamma, 1e-4
    g = lvl.grad(v, lam, gam)[0]
    u = v.copy()
    S = np.zeros(len(O.FIELDS))
    S[O.K["lam"]], S[O.K["gam"]], S[O.K["alpha"]], S[O.K["a"]], S[O.K["mu"]] = lam, gam, 1.0, 1.0, 1.0
    S[O.K["best_hpwl"]] = S[O.K["best_ovf"]] = math.inf
    kp = np.array([gam, lam, lam, 1.0, 0.0], np.float32)
    c = prob.constants()
    t0 = None
    for k in range(iters + 2):
        if k == 2:
            t0 = time.time()
        un, vn = O.nesterov_step(u, v, g, gr.pos_lo, gr.pos_hi, kp[3], kp[4])
        gn, wa, hpwl, ovf = lvl.grad(vn, float(kp[1]), float(kp[0]))
        O.control(S, kp, c, np.linalg.norm(vn - v), np.linalg.norm(gn - g), hpwl, ovf, wa)
        u, v, g = un, vn, gn
    return (time.time() - t0) / iters, threads


def cpu_baseline_dict(per, threads, iters, gpu_iters):
    return {"value": round(per * gpu_iters, 3), "unit": "s", "cores": threads, "kind": "port",
            "sample": "%d density-phase iterations of the oracle's CPU iteration (the reference's --gpu -1 path "
                      "restated: float32 operators, FFT field) on the cells of the full netlist, on %d host threads: "
                      "%.4f s/iter x the %d iterations of this GB300 placement (a bounded sample; bench.py --impl "
                      "reference runs the CPU placement to its own stop)" % (iters, threads, per, gpu_iters)}


# ------------------------------------------------------------------------------------------------ roofline
def kernel_bytes(prob, field="f16x3"):
    """Algorithmic bytes (or flops) per launch of each kernel, by launcher name."""
    terms = 3 if field in ("bf16x6", "bf16x3") else 2 if field == "f16x3" else 0     # 16-bit density terms out
    dens = 8 if field == "tf32x3" else 2 * terms if terms else 4                      # (tf32x3: 2 float32 terms)
    cs, n, c = prob.csr, prob.num_nodes, prob.num_mov
    P, N = len(cs.cell32), cs.num_nets
    nb = prob.force_bin * prob.force_bin
    jn = prob.num_bin * prob.num_bin if prob.judge is not None else 0
    return {
        "launch_wa_net": 20 * P + 8 * c + 4 * N,                       # pins (cell, offset) in, pin gradient out
        "launch_gather": 44 * n + 12 * P + 4 * c + 8 * nb,             # node data, cell CSR gather, field planes
        "launch_scatter": 20 * n + 16 * nb,                            # node data in, map out (force grid); judge below
        "launch_post_plain": (36 + dens) * nb,                          # map in + zeroed, fixed in, density terms out
        "launch_step": 56 * n,                                          # u, v, g, lo, hi in; u', v' out
    }


def tc_flops(prob, field):
    """Tensor-core FLOPs of the field per density pass: six GEMMs of nb^3 (2 nb^3 per product, the mode's products
    each); f16x3 on a grid of a multiple of 256 bins folds the transforms: each forward one into two GEMMs of half
    the height and half the depth, each inverse one into half-height products that also give the mirror rows -- half
    the products in all."""
    nb = prob.force_bin
    terms = {"bf16x6": 6, "bf16x3": 3, "f16x3": 3, "tf32x3": 3}.get(field, 0)
    gemms = 3.0 if field == "f16x3" and nb % 256 == 0 else 6.0
    return 2.0 * nb ** 3 * terms * gemms


def profile_pass(placer):
    """Per-launch durations of one density pass (eager, CUDA events on the engine's stream), averaged over 8."""
    from autoplace_gb300 import native
    # one stream (the split pass runs the WA kernels beside the density map: per-launch events would overlap)
    rec = native.profile(placer.stream.cuda_stream, lambda: placer._passes(native.PHASE_DENSITY, 8, split=False))
    agg = {}
    for name, ms in rec:
        a = agg.setdefault(name, [0, 0.0])
        a[0] += 1
        a[1] += ms
    return {k: {"launches_per_pass": v[0] / 8.0, "ms_per_pass": v[1] / 8.0} for k, v in agg.items()}, rec


def measured_traffic(config, field):
    """DRAM bytes (read + write) per pass of each launcher, from the committed ncu summary of this workload."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_%s.json" % config)) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return {}
    return rec["bytes"] if rec.get("field") == field else {}


def roofline(prob, field, prof, peaks, config="c2"):
    traffic = measured_traffic(config, field)
    hbm = peaks.get("hbm_gbs")
    tc = peaks.get("bf16_tflops")
    by = kernel_bytes(prob, field)
    dom = max(prof.items(), key=lambda kv: kv[1]["ms_per_pass"])
    name, d = dom
    ms_launch = d["ms_per_pass"] / max(d["launches_per_pass"], 1e-9)
    table = {}
    for k, v in prof.items():
        ml = v["ms_per_pass"] / max(v["launches_per_pass"], 1e-9)
        row = {"ms_per_pass": round(v["ms_per_pass"], 4), "launches_per_pass": v["launches_per_pass"],
               "ms_per_launch": round(ml, 4)}
        if k in by:     # algorithmic bytes of the whole pass over the kernel's time per pass (all its launches)
            row["gbs"] = round(by[k] / (v["ms_per_pass"] * 1e-3) / 1e9, 1)
        if k == "launch_tc_mode":
            f = tc_flops(prob, field) / v["launches_per_pass"]
            row["tflops"] = round(f / (ml * 1e-3) / 1e12, 1)
        table[k] = row
    if name == "launch_tc_mode":
        f = tc_flops(prob, field) / d["launches_per_pass"]
        ach = f / (ms_launch * 1e-3) / 1e12
        r = {"kernel": "tc_gemm_kernel", "bound": "tensor", "achieved": round(ach, 1), "peak": tc,
             "unit": "TFLOP/s", "frac": round(ach / tc, 4) if tc else None, "traffic": traffic.get(name),
             "peak_source": "measured (MEASURED_PEAKS.json bf16_tflops)"}
    else:
        b = by.get(name)
        ach = b / (d["ms_per_pass"] * 1e-3) / 1e9 if b else None
        r = {"kernel": name, "bound": "hbm", "achieved": round(ach, 1) if ach else None, "peak": hbm, "unit": "GB/s",
             "frac": round(ach / hbm, 4) if ach and hbm else None,
             "traffic": round(traffic[name] / max(d["launches_per_pass"], 1e-9)) if name in traffic else None,
             "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)"}
    return r, table


def native_modes():
    from autoplace_gb300 import native
    return native.FIELD_MODES


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# ------------------------------------------------------------------------------------------------ arms
def _start_hook(args, prob):
    """The clusters' start of the product's configuration -> (hook for Flow.run or None, name, the learned hook when
    a model exists (measured beside the line even when the fallback rule keeps the plain start))."""
    from autoplace_gb300 import learn
    prop = learn.Proposal(learn.load_model()) if os.path.exists(learn.MODEL_FILE) else None
    if args.start == "plain" or prop is None:
        return None, "plain (wirelength-only)", prop
    if args.start == "learned":
        return prop.hook, "learned (message-passing proposal of the cluster positions)", prop
    if not learn.model_available():
        return None, "plain (wirelength-only; the model did not pass its validation)", prop
    if not prop.applies(prob):
        return None, ("plain (wirelength-only): fallback, %d cells is outside the %d-%d cells the learned start was "
                      "trained and validated on" % (prob.num_mov, prop.cells[0], prop.cells[1])), prop
    return prop.hook, "learned (message-passing proposal of the cluster positions)", prop


def _timed_runs(flow, pos, steps, start=None):
    """`steps` placements, CUDA events on the flow's stream around them -> (seconds per placement, last stats, wall)."""
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(flow.stream)
    t0 = time.time()
    st = None
    for _ in range(steps):
        st = flow.run(pos, start=start)
    ev1.record(flow.stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1000.0 / max(steps, 1), st, time.time() - t0


def run_gb300(args):
    import numpy as np
    import torch
    from autoplace_gb300 import engine
    from autoplace_gb300.flow import Flow
    rank, world, local = dist_setup()
    if args.no_pdl:
        from autoplace_gb300 import native
        native.call("gp103_set_option", 0, 0)
    prob, pos0 = workload(args.config, seed=rank)
    start, start_name, prop = _start_hook(args, prob)
    flow = Flow(prob, field=args.field)
    dpos = torch.tensor(pos0, device="cuda")
    for _ in range(max(args.warmup, 0)):
        flow.run(dpos, start=start)
    torch.cuda.synchronize()
    barrier(world)
    clocks = Clocks(local)
    clocks.start()
    l0 = engine.launches()
    step_s, last, wall = _timed_runs(flow, dpos, args.steps, start)
    launches = engine.launches() - l0
    barrier(world)
    clk = clocks.stop()
    step_s = reduce_max(step_s, world)
    iters = last["iters"]
    hpwl_exact, overflow_exact = flow.fine.evaluate(last["pos"])
    result = {"stop": last["stop_reason"], "fallback": bool(last.get("fallback", False)),
              "iterations": iters, "start_iterations": last["start_iters"],
              "clusters": last.get("clusters"), "cluster_iterations": last.get("coarse_iters"),
              "hpwl_exact": hpwl_exact, "overflow": last["overflow"], "overflow_exact": overflow_exact,
              "ms_per_iteration": round(step_s * 1000 / max(iters, 1), 4), "phase_s": last.get("phase_s"),
              "wall_s_per_step": round(wall / max(args.steps, 1), 4)}

    # the plain method on the same GPU: the reference's start (wirelength-only) and a float32 field
    plain = None
    if not args.no_plain:
        pflow = Flow(prob, field=args.plain_field)
        pflow.run(dpos)                                                     # warm-up (graphs, set-up)
        p_s, pst, _ = _timed_runs(pflow, dpos, args.plain_steps)
        ph, po = pflow.fine.evaluate(pst["pos"])
        plain = {"value": round(p_s, 4), "unit": "s", "field": args.plain_field, "start": "plain (wirelength-only)",
                 "stop": pst["stop_reason"], "iterations": pst["iters"], "hpwl_exact": ph, "overflow": pst["overflow"],
                 "overflow_exact": po, "steps": args.plain_steps}
        result["speedup_vs_plain"] = round(p_s / step_s, 3)
        result["hpwl_vs_plain"] = round(hpwl_exact / ph, 5)
        del pflow
        if start is None and prop is not None:
            # the learned start measured beside the line (the fallback rule kept the plain start)
            flow.run(dpos, start=prop.hook)
            l_s, lst, _ = _timed_runs(flow, dpos, args.plain_steps, prop.hook)
            lh, lo = flow.fine.evaluate(lst["pos"])
            result["learned_start"] = {"value": round(l_s, 4), "iterations": lst["iters"], "hpwl_exact": lh,
                                       "overflow_exact": lo, "vs_this_line": round(l_s / step_s, 3),
                                       "hpwl_vs_this_line": round(lh / hpwl_exact, 5),
                                       "proposal_s": lst.get("phase_s", {}).get("proposal")}
        if start is not None:
            # the learned start's own share: the same tensor-core field with the plain start
            flow.run(dpos)
            t_s, tst, _ = _timed_runs(flow, dpos, args.plain_steps)
            th, to = flow.fine.evaluate(tst["pos"])
            plain["tc_plain_start"] = {"value": round(t_s, 4), "iterations": tst["iters"], "hpwl_exact": th,
                                       "overflow_exact": to}
            result["speedup_vs_tc_plain_start"] = round(t_s / step_s, 3)

    # e2e: from the netlist's pinned host arrays through the public API: upload, the problem's arrays built on the
    # device (net CSR, cell order, smoothed nodes), the cells' Placer and the flow (the clustering reads the problem's
    # pins on the device), the run, the download of the placement. The host part of the problem (grids, fixed
    # fractions, fillers: the reader's and initializer's work) is made once, before.
    from autoplace_gb300.problem import Problem, netlist_arrays
    base = Problem(prob.nl, prob.opts, arrays=False)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    host = {k: pin(v) for k, v in netlist_arrays(base).items()}
    maps = {"fixed": pin(base.force.fixed_map)}
    if base.judge is not None:
        maps["jfixed"] = pin(base.judge.fixed_map)
    host_pos = pin(np.asarray(pos0, dtype=np.float32))
    out = torch.empty(host_pos.shape, dtype=torch.float32).pin_memory()
    h2d = sum(x.numel() * x.element_size() for x in list(host.values()) + list(maps.values())) + \
        host_pos.numel() * 4 + len(prob.constants()) * 8
    d2h = out.numel() * 4
    # one untimed step first: it loads the device-build kernels, which only this path uses (a one-time cost per
    # process, like the warm-up placements of the device-timed loop)
    e2e_s = []
    for i in range(1 + args.e2e_steps):
        torch.cuda.synchronize()
        t = time.time()
        dprob = base.on_device(stream=flow.stream, host=host)
        f2 = Flow(dprob, field=args.field, stream=flow.stream, host=maps)
        rr = f2.run(host_pos, start=start)
        out.copy_(rr["pos"])
        torch.cuda.synchronize()
        if i > 0:
            e2e_s.append(time.time() - t)
        del f2, dprob, rr
    e2e = reduce_max(statistics.median(e2e_s), world)

    prof, _ = profile_pass(flow.fine)
    peaks = load_peaks()
    roof, table = roofline(prob, args.field, prof, peaks, args.config)
    ctable = None
    if flow.last_coarse is not None:
        # the clusters' level too: one more placement keeping its Placer, profiled at the state it handed over at
        flow.keep_coarse_placer = True
        flow.run(dpos, start=start)
        flow.keep_coarse_placer = False
        cpl = flow.last_cplacer
        if cpl is not None:
            cprof, _ = profile_pass(cpl)
            cfield = {v: k for k, v in native_modes().items()}.get(cpl.mode, args.field)
            ctable = roofline(cpl.p, cfield, cprof, peaks, "none")[1]
        flow.last_cplacer = None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        per, threads = cpu_sample(prob, pos0, args.cpu_iters)
        cpu = cpu_baseline_dict(per, threads, args.cpu_iters, iters)
    line = {"metric": METRIC, "value": round(step_s, 4), "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(step_s * 1000, 2), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (field: %s tensor cores; f64 reductions)" % args.field,
            "data": "synthetic (seeded generator standing in for ISPD 2015/2019)",
            "config": config_dict(prob, args, world, start_name), "result": result, "plain": plain,
            "e2e": {"value": round(e2e, 4), "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": roof, "kernels": table, "kernels_clusters": ctable, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": int(launches)}
    if rank == 0:
        print(json.dumps(line))


def run_batch(args):
    """--config c3: 64 uneven instances (5k-150k cells, grids 64-512, 0-10 macros), tuned per size class, placed as
    one batch (one CUDA graph) and one by one; aggregate iterations/s and p50 / p99 time to the stop."""
    import numpy as np
    import torch
    from autoplace_gb300 import engine, problem, synth, tune
    from autoplace_gb300.batch import Batch
    from autoplace_gb300.engine import Placer
    rank, world, local = dist_setup()
    t_setup = time.time()
    probs, pos = [], []
    for nl, o in synth.batch_instances(count=args.instances, seed=rank):
        pr = problem.Problem(nl, problem.options(**o))
        probs.append(pr)
        pos.append(synth.init_positions(nl, pr.num_nodes, seed=1))
    host_s = time.time() - t_setup
    t_tune = time.time()
    tuned = [tune.tune(p, p0) for p, p0 in zip(probs, pos)]
    tune_s = time.time() - t_tune
    b = Batch(probs, tuned=tuned)
    for _ in range(max(args.warmup, 1)):
        b.run(pos)
    clocks = Clocks(local)
    clocks.start()
    l0 = engine.launches()
    walls, pers, res = [], [], None
    for _ in range(args.steps):
        res, per, wall = b.run(pos)
        walls.append(wall)
        pers.append(per)
    launches = engine.launches() - l0
    clk = clocks.stop()
    iters = sum(r["iters"] for r in res)
    wall = reduce_max(statistics.median(walls), world)
    per = np.median(np.stack(pers), 0)
    # one by one, the same tuned settings, each Placer set up once (warm-up run first)
    singles = []
    for p, p0, t in zip(probs, pos, tuned):
        pl = Placer(p, field=t["field"])
        tune.apply_wa(pl, t["wa"])
        pl.run(p0)
        torch.cuda.synchronize()
        t0 = time.time()
        pl.run(p0)
        torch.cuda.synchronize()
        singles.append(time.time() - t0)
        del pl
    single_total = float(np.sum(singles))
    line = {"metric": "aggregate iterations/s, batch of %d uneven instances in one CUDA graph"
                      % len(probs),
            "value": round(iters / wall, 1), "unit": "iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(wall * 1000, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (field per instance: tuned; f64 reductions)",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "synthetic c3: %d instances, cells log-uniform 5k-150k (%d .. %d), nets 1.05x, "
                                   "0-10 macros, grids %d .. %d, one level each"
                                   % (len(probs), min(p.num_mov for p in probs), max(p.num_mov for p in probs),
                                      min(p.force.nbx for p in probs), max(p.force.nbx for p in probs)),
                       "instances": len(probs), "graphs_per_batch": 1},
            "result": {"iterations": iters, "batch_s": round(wall, 4),
                       "time_to_stop_p50_s": round(float(np.percentile(per, 50)), 4),
                       "time_to_stop_p99_s": round(float(np.percentile(per, 99)), 4),
                       "one_by_one_s": round(single_total, 4),
                       "one_by_one_iter_per_s": round(iters / single_total, 1),
                       "one_by_one_p50_s": round(float(np.percentile(singles, 50)), 4),
                       "one_by_one_p99_s": round(float(np.percentile(singles, 99)), 4),
                       "speedup_vs_one_by_one": round(single_total / wall, 3),
                       "stops": sorted(set(r["reason"] for r in res)),
                       "tuned": {k: sum(1 for t in tuned if "%s/%s" % (t["field"], t["wa"]) == k)
                                 for k in set("%s/%s" % (t["field"], t["wa"]) for t in tuned)},
                       "host_setup_s": round(host_s, 2), "tune_s": round(tune_s, 2)},
            "clocks": clk, "gpu_launches": int(launches)}
    if rank == 0:
        print(json.dumps(line))


def _cpu_judges(prob, pos):
    """Exact HPWL over every net and the movable cells' overflow with their real sizes (float64, the oracle)."""
    import numpy as np
    from oracle import gp_oracle as O
    gr, C = prob.real_judge, prob.num_mov
    pos = np.asarray(pos, np.float32)
    hpwl = O.hpwl_all(pos, prob.all_cell, prob.all_off, prob.all_net_start, C)
    size = np.ascontiguousarray(prob.nl.size, dtype=np.float32)
    m = O.density_map_mt(pos[:C], size, np.ones(C, np.float32), C, gr.bx, gr.by, gr.nbx, gr.nby)
    _, _, total = O.density_post(m, gr.fixed_map, gr.target, gr.nbx, gr.nby, mirrored=False)
    return float(hpwl), float(total * gr.bin_area / gr.mov_area)


def run_reference(args):
    """The reference's CPU path (restated by the oracle: float32 operators, FFT of the mirrored map) on every host
    core: W untimed gradient evaluations, then one whole placement of the same netlist and flow (two levels at the
    reference's default cluster ratio) to its own stop, timed in full."""
    rank, world, _ = dist_setup()
    if rank != 0:
        return
    import numpy as np
    from oracle import gp_oracle as O
    prob, pos0 = workload(args.config, seed=0)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    lvl = O.CpuLevel(prob, dtype=np.float32, field="fft", threads=threads)
    gr = prob.force
    v = np.clip(np.asarray(pos0, np.float64), gr.pos_lo, gr.pos_hi)
    for _ in range(max(args.warmup, 0)):
        lvl.grad(v, 1e-4, 10 * prob.base_gamma)
    t0 = time.time()
    if prob.opts.cluster_ratio > 1:
        r = O.two_level(prob, pos0, dtype=np.float32, field="fft", threads=threads)
        extra = {"clusters": r["clusters"], "cluster_iterations": r["coarse_iters"]}
    else:
        r = O.CpuLevel(prob, dtype=np.float32, field="fft", threads=threads).run(pos0)
        extra = {}
    total = time.time() - t0
    hpwl, ovf = _cpu_judges(prob, r["pos"])
    steps = max(args.steps, 1)
    cpu = {"value": round(total, 3), "unit": "s", "cores": threads, "kind": "port",
           "sample": "one whole placement to its own stop (%s, %d iterations), timed in full on %d host threads; "
                     "the %d steps are consecutive shares of it" % (r["reason"], r["iters"], threads, steps)}
    line = {"impl": "reference", "metric": METRIC, "value": round(total, 3), "unit": "s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": round(total * 1000 / steps, 1),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 operators, f64 control (CPU)",
            "data": "synthetic (seeded generator standing in for ISPD 2015/2019)",
            "config": config_dict(prob, args, world, "plain (wirelength-only)"),
            "result": dict(stop=r["reason"], iterations=r["iters"], hpwl_exact=hpwl, overflow=r["overflow"],
                           overflow_exact=ovf, **extra),
            "cpu_baseline": cpu,
            "e2e": {"value": round(total, 3), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["config"]["field"] = "fft (float32, mirrored map)"
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == "c3":
        run_batch(a)
    else:
        run_gb300(a)
