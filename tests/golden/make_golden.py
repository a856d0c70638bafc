"""Generate the golden fixtures of tests/golden/ from AutoPlace's own PyTorch operators (its CPU path).

Run with the path of a checkout of the AutoPlace sources (an argument, or $AUTOPLACE_REF):

    python tests/golden/make_golden.py <autoplace checkout>

It imports the reference with its compiled modules absent (gp_cuda = None), i.e. exactly the `--gpu -1` code path,
feeds it seeded synthetic inputs from autoplace_gb300.synth, and stores inputs and outputs as small .npz files. The
tests read only these files: the reference sources are not needed to run them.

  golden_wa.npz        Wirelength: CSR of the optimised nets (kernel view), WA / grad / HPWL at two gammas, exact HPWL
  golden_density.npz   ElectronicDensityLayer: smoothing, mirrored density + overflow, field, forward gradient,
                       exact / smoothed overflow on a second (overflow) grid
  golden_control.npz   ParamScheduler + resolution: the state after each step of a driven sequence
  golden_place.npz     global_placement_main (one level) on a small netlist: stop reason, iterations, HPWL, overflow
  golden_cluster.npz   cluster_cells: the merged pair edges, the head draws and edges of every round, the clusters
  golden_coarse.npz    coarse_problem + expand: the cluster problem (sizes, pins, grid) and the expanded positions
  golden_place2.npz    global_placement_main with two levels (cluster_ratio 5) on a small netlist
"""
import math
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AUTOPLACE_REF")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("usage: python tests/golden/make_golden.py <path of the AutoPlace sources> (or set AUTOPLACE_REF)")
sys.path.insert(0, REPO)
sys.path.insert(0, REF)

import torch  # noqa: E402

from autoplace_gb300 import synth, problem  # noqa: E402
import cpp_to_py  # noqa: E402

assert cpp_to_py.gp_cuda is None, "the golden fixtures come from the PyTorch operators: gp_cuda must not be built"
from src.core import ElectronicDensityLayer, Wirelength  # noqa: E402
from src import param_scheduler, run_placement  # noqa: E402

torch.set_num_threads(4)


def small_netlist(seed, cells=600, nets=650, macros=3, cover=0.12):
    nl = synth.make_netlist(cells, nets, window=40, macros=macros, cover=cover, fixed_pin_share=0.08, seed=seed)
    # one net of degree 1 and one above ignore_net_degree (both left out of the optimised set)
    extra_cells = np.arange(0, 130) % cells
    pin_cell = np.concatenate([nl.pin_cell, [5], extra_cells])
    pin_off = np.concatenate([nl.pin_off, [[0.1, -0.2]], np.zeros((len(extra_cells), 2))])
    pin_net = np.concatenate([nl.pin_net, [nl.num_nets], np.full(len(extra_cells), nl.num_nets + 1)])
    nl.pin_cell, nl.pin_off, nl.pin_net, nl.num_nets = pin_cell.astype(np.int64), pin_off, pin_net.astype(np.int64), nl.num_nets + 2
    return nl


def gen_wa():
    nl = small_netlist(11)
    n = nl.num_mov
    t = lambda a, dt: torch.tensor(a, dtype=dt)
    wl = Wirelength(t(nl.pin_cell, torch.long), t(nl.pin_off, torch.float32), t(nl.pin_net, torch.long), nl.num_nets,
                    n, 100)
    kview = Wirelength._pin_set(SimpleNamespace(kernel=True, num_mov=n), t(nl.pin_cell, torch.long)[wl_sel(nl)],
                                t(nl.pin_off, torch.float32)[wl_sel(nl)], renumber(nl), wl.num_opt_nets)
    rng = np.random.default_rng(3)
    pos = (rng.random((n + 40, 2)) * [nl.width, nl.height]).astype(np.float32)
    out = dict(pin_cell=nl.pin_cell, pin_off=nl.pin_off.astype(np.float32), pin_net=nl.pin_net, num_nets=nl.num_nets,
               num_mov=n, ignore_net_degree=100, pos=pos,
               net_start=kview["net_start"].numpy(), cell_start=kview["cell_start"].numpy(),
               cell_pin=kview["cell_pin"].numpy(), cell32=kview["cell32"].numpy(), off_opt=kview["off"].numpy())
    for k, gamma in enumerate([4.0, 0.37]):
        wa, grad, hpwl = wl.forward(torch.tensor(pos), gamma)
        out["gamma%d" % k] = gamma
        out["wa%d" % k], out["grad%d" % k], out["hpwl%d" % k] = float(wa), grad.numpy(), float(hpwl)
    out["hpwl_all"] = float(wl.hpwl(torch.tensor(pos)))
    np.savez_compressed(os.path.join(HERE, "golden_wa.npz"), **out)


def wl_sel(nl):
    deg = np.bincount(nl.pin_net, minlength=nl.num_nets)
    use = (deg >= 2) & (deg <= 100)
    return torch.tensor(use[nl.pin_net])


def renumber(nl):
    deg = np.bincount(nl.pin_net, minlength=nl.num_nets)
    use = (deg >= 2) & (deg <= 100)
    new_id = np.cumsum(use) - 1
    return torch.tensor(new_id[nl.pin_net[use[nl.pin_net]]])


def gen_density():
    nl = small_netlist(12, cells=900, nets=950)
    opts = problem.options(target_density=0.9, num_bin=16, force_num_bin=32)
    prob = problem.Problem(nl, opts)
    n = nl.num_mov
    ff = nl.fixed_fraction(32, 32)
    jf = nl.fixed_fraction(16, 16)
    layer = ElectronicDensityLayer(nl.width, nl.height, 32, 32, ff, prob.target, prob.node_size, n, "cpu",
                                   np.concatenate([nl.cell_pins, np.zeros(prob.num_nodes - n)]))
    layer.judge = ElectronicDensityLayer(nl.width, nl.height, 16, 16, jf, prob.target, nl.size, n, "cpu", field=False)
    rng = np.random.default_rng(5)
    pos = torch.tensor(rng.random((prob.num_nodes, 2)) * [nl.width, nl.height], dtype=torch.float32)
    pos = torch.max(torch.min(pos, layer.pos_hi), layer.pos_lo)
    # a clump: the first 100 cells near one point (many nodes per bin)
    pos[:100] = pos[:100] * 0.02 + torch.tensor([nl.width * 0.3, nl.height * 0.6])
    pos = torch.max(torch.min(pos, layer.pos_hi), layer.pos_lo)
    mirrored, ovf_force = layer._density(pos, layer.smooth, n)
    field = torch.fft.irfft2(torch.fft.rfft2(mirrored) * layer.to_field, s=(64, 64))
    wl_grad = torch.tensor(rng.standard_normal((n, 2)), dtype=torch.float32)
    grad, ovf = layer.forward(pos, wl_grad, 0.37, 0.37)
    plain, _ = layer.forward(pos)
    out = dict(width=nl.width, height=nl.height, target=prob.target, num_mov=n, node_size=prob.node_size,
               fixed_fraction=ff, judge_fraction=jf, pos=pos.numpy(),
               smooth_size=layer.smooth["size"].numpy(), smooth_ratio=layer.smooth["ratio"].numpy(),
               pos_lo=layer.pos_lo.numpy(), pos_hi=layer.pos_hi.numpy(), fixed_map=layer.fixed_map.numpy(),
               pins=layer.pins.numpy(), area=layer.area.numpy(),
               judge_size=layer.judge.smooth["size"].numpy(), judge_ratio=layer.judge.smooth["ratio"].numpy(),
               mirrored=mirrored.numpy(), overflow_force=float(ovf_force), field=field.numpy(),
               wl_grad=wl_grad.numpy(), grad=grad.numpy(), overflow=float(ovf), plain_grad=plain.numpy(),
               exact_overflow=float(layer.exact_overflow(pos[:n].contiguous())),
               to_field=layer.to_field.numpy())
    # The reference's CPU rasteriser folds the part of a node beyond the upper region edge into the last bin, its
    # CUDA kernel drops it. Nodes smoothed on the coarser overflow grid can reach past the edge, so the overflow-grid
    # check uses positions kept inside that grid's own bounds, where both paths agree.
    jlo = layer.judge.smooth["size"] / 2
    jpos = torch.max(torch.min(pos[:n], torch.tensor([nl.width, nl.height]) - jlo), jlo).contiguous()
    out["judge_pos"] = jpos.numpy()
    out["judge_overflow"] = float(layer.judge.smoothed_overflow(jpos))
    out["judge_exact_overflow"] = float(layer.exact_overflow(jpos))
    np.savez_compressed(os.path.join(HERE, "golden_density.npz"), **out)


def gen_control():
    """Drive ParamScheduler with a seeded sequence and record its state after every step."""
    args = SimpleNamespace(wa_coeff=4.0, wa_rule="accuracy", start_tol=1e-3, min_iter=20, stop_overflow=0.07,
                           settle_iter=10, stall_iter=15)
    rows, rules = [], []
    for rule in ("accuracy", "overflow"):
        args.wa_rule = rule
        data = SimpleNamespace(bin=np.array([3.7, 4.1]), total_pins=5000.0, total_area=81234.5, num_nodes=1800,
                               pitch=2.9, refine=2.0)
        ps = param_scheduler.ParamScheduler(data, args, None)
        ps.density_weight = 1.3e-4
        ps.hpwl.append(1.0e6)
        ps.iter = 7
        rng = np.random.default_rng(17 if rule == "accuracy" else 18)
        hpwl, ovf = 1.0e6, 0.9
        for k in range(120):
            hpwl *= float(np.exp(rng.normal(0.002, 0.01)))
            ovf = max(0.0, ovf * float(np.exp(rng.normal(-0.03, 0.04))))
            moved = float(rng.uniform(10, 400))
            wa = hpwl * float(rng.uniform(0.7, 0.99))
            ps.step(hpwl, ovf, moved, wa)
            reason = ps.need_to_stop()
            code = {None: 0, "converged": 1, "stalled": 2, "diverged": 3, "handover": 5}[reason]
            rows.append([k, hpwl, ovf, moved, wa, ps.density_weight, ps.wa_coeff, ps.mu, ps.motion, ps.weighted_weight,
                         ps.settled, ps.best_hpwl, ps.best_overflow, float(ps.is_best), ps.improved_iter, ps.iter, code])
            rules.append(rule == "accuracy")
            if reason:
                break
    np.savez_compressed(os.path.join(HERE, "golden_control.npz"), rows=np.array(rows), accuracy=np.array(rules),
                        base_gamma=4.0 * (3.7 + 4.1), lam0=1.3e-4, hpwl0=1.0e6, iter0=7, total_pins=5000.0,
                        total_area=81234.5, num_nodes=1800, pitch=2.9, refine=2.0, min_iter=20, stop_overflow=0.07,
                        settle_iter=10, stall_iter=15)


class _Log(object):
    def info(self, *_):
        pass


def gen_place():
    nl = synth.make_netlist(2500, 2620, window=80, macros=0, seed=21)
    opts = problem.options(target_density=1.0, num_bin=32, force_num_bin=0, cluster_ratio=1.0, inner_iter=3000)
    prob = problem.Problem(nl, opts)
    n = nl.num_mov
    t = lambda a, dt: torch.tensor(a, dtype=dt)
    wl = Wirelength(t(nl.pin_cell, torch.long), t(nl.pin_off, torch.float32), t(nl.pin_net, torch.long), nl.num_nets,
                    n, opts.ignore_net_degree)
    density = ElectronicDensityLayer(nl.width, nl.height, prob.force_bin, prob.force_bin, nl.fixed_fraction(prob.force_bin, prob.force_bin),
                                     prob.target, prob.node_size, n, "cpu",
                                     np.concatenate([nl.cell_pins, np.zeros(prob.num_nodes - n)]))
    if prob.force_bin != prob.num_bin:                 # the overflow grid, as run_placement_main sets it up
        density.judge = ElectronicDensityLayer(nl.width, nl.height, prob.num_bin, prob.num_bin,
                                               nl.fixed_fraction(prob.num_bin, prob.num_bin), prob.target, nl.size, n,
                                               "cpu", field=False)
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    pos = torch.tensor(pos0)
    data = SimpleNamespace(num_mov=n, mov_area=nl.mov_area, cell_pins=nl.cell_pins)
    args = SimpleNamespace(**vars(opts))
    stats = run_placement.global_placement_main(data, wl, density, pos, prob.node_size, None, args, _Log())
    hpwl = float(wl.hpwl(pos))
    ovf = float(density.exact_overflow(pos[:n].contiguous()))
    np.savez_compressed(os.path.join(HERE, "golden_place.npz"), pos0=pos0, cells=2500, nets=2620, window=80, seed=21,
                        num_bin=32, force_bin=prob.force_bin, iters=stats["iters"], start_iters=stats["start_iters"],
                        reason=stats["stop_reason"], hpwl=hpwl, overflow=ovf, grad_calls=stats["grad_calls"])
    print("place:", stats["stop_reason"], stats["iters"], stats["start_iters"], hpwl, ovf)


def gen_cluster():
    """cluster_cells on a netlist with fixed pins, nets above max_degree and a few cells above 20 x the mean area.
    The edges are read from the reference's own _merge_edges (after the pair loop, and after every round) and the
    head draws from torch.rand, so that a restatement can be checked step by step."""
    from src import cluster as C
    nl = synth.make_netlist(4000, 4300, window=120, macros=3, cover=0.1, fixed_pin_share=0.05, seed=31)
    size = nl.size.copy()
    size[[7, 1500, 3333], 0] *= 400                      # three cells above 20 x the mean area
    area = np.round(size.prod(1) * 1024).astype(np.int64)
    ratio, seed = 5, 17
    calls, draws = [], []
    merge, rand = C._merge_edges, torch.rand

    def spy_merge(parts, n):
        r = merge(parts, n)
        calls.append([x.numpy().copy() for x in r])
        return r

    def spy_rand(*a, **k):
        r = rand(*a, **k)
        draws.append(r.numpy().copy())
        return r

    C._merge_edges, C.torch.rand = spy_merge, spy_rand
    try:
        cid, carea = C.cluster_cells(torch.tensor(nl.pin_cell), torch.tensor(nl.pin_net), torch.tensor(area), ratio, seed)
    finally:
        C._merge_edges, C.torch.rand = merge, rand
    out = dict(pin_cell=nl.pin_cell, pin_net=nl.pin_net, area=area, ratio=ratio, seed=seed, n=nl.num_mov,
               edge_i=calls[6][0], edge_j=calls[6][1], edge_w=calls[6][2], rounds=len(draws),
               cid=cid.numpy(), carea=carea.numpy())
    for r, d in enumerate(draws):
        out["draw%d" % r] = d
        if 7 + r < len(calls):
            out["round%d_i" % r], out["round%d_j" % r], out["round%d_w" % r] = calls[7 + r]
    np.savez_compressed(os.path.join(HERE, "golden_cluster.npz"), **out)
    print("cluster:", nl.num_mov, "cells ->", len(carea), "clusters in", len(draws), "rounds;", len(calls[6][0]), "edges")


def _ref_problem(nl, opts):
    """The reference's objects for a netlist, as run_placement_main builds them (CPU operators)."""
    prob = problem.Problem(nl, opts)
    n = nl.num_mov
    t = lambda a, dt: torch.tensor(a, dtype=dt)
    wl = Wirelength(t(nl.pin_cell, torch.long), t(nl.pin_off, torch.float32), t(nl.pin_net, torch.long), nl.num_nets,
                    n, opts.ignore_net_degree)
    ff = nl.fixed_fraction(prob.force_bin, prob.force_bin)
    density = ElectronicDensityLayer(nl.width, nl.height, prob.force_bin, prob.force_bin, ff, prob.target,
                                     prob.node_size, n, "cpu", np.concatenate([nl.cell_pins, np.zeros(prob.num_nodes - n)]))
    if prob.force_bin != prob.num_bin:
        density.judge = ElectronicDensityLayer(nl.width, nl.height, prob.num_bin, prob.num_bin,
                                               nl.fixed_fraction(prob.num_bin, prob.num_bin), prob.target, nl.size, n,
                                               "cpu", field=False)
    data = SimpleNamespace(num_mov=n, mov_area=nl.mov_area, cell_pins=nl.cell_pins, width=nl.width, height=nl.height,
                           fixed_fraction=nl.fixed_fraction)
    return prob, wl, density, ff, data


def gen_coarse():
    """coarse_problem (src/cluster.py:88-130) and expand (:133-144) on a netlist with macros and fixed pins."""
    from src import cluster as C
    nl = synth.make_netlist(3000, 3200, window=100, macros=3, cover=0.1, fixed_pin_share=0.05, seed=41)
    opts = problem.options(target_density=0.9, num_bin=32, force_num_bin=64, cluster_ratio=4.0, seed=3)
    prob, wl, density, ff, data = _ref_problem(nl, opts)
    args = SimpleNamespace(**vars(opts))
    coarse = C.coarse_problem(data, prob.node_size, wl, density, ff, args)
    cw = coarse.wirelength.all
    rng = np.random.default_rng(9)
    cpos = torch.tensor(rng.random((coarse.num_nodes, 2)) * [nl.width, nl.height], dtype=torch.float32)
    pos = C.expand(cpos, coarse, prob.node_size, opts.seed)
    cd = coarse.density
    np.savez_compressed(os.path.join(HERE, "golden_coarse.npz"), seed=41, cells=3000, nets=3200, window=100, macros=3,
                        cover=0.1, fixed_pin_share=0.05, target_density=0.9, num_bin=32, force_num_bin=64,
                        cluster_ratio=4.0, cluster_seed=3,
                        cid=coarse.cid.numpy(), num=coarse.num, size=coarse.size.numpy(),
                        pin_cell=cw["cell"].numpy(), pin_off=cw["off"].numpy(), pin_net=cw["net"].numpy(),
                        num_nets=cw["num_nets"], nbx=cd.nbx, smooth_size=cd.smooth["size"].numpy(),
                        smooth_ratio=cd.smooth["ratio"].numpy(), pins=cd.pins.numpy(), fixed_map=cd.fixed_map.numpy(),
                        total_pins=coarse.total_pins, total_area=coarse.total_area, num_nodes=coarse.num_nodes,
                        cpos=cpos.numpy(), pos=pos.numpy())
    print("coarse:", coarse.num, "clusters,", cd.nbx, "bins,", len(cw["cell"]), "pins")


def gen_place2():
    """The two-level run: clusters placed first (until the hand-over smoothing), then the cells."""
    nl = synth.make_netlist(2500, 2620, window=80, macros=0, seed=21)
    opts = problem.options(target_density=1.0, num_bin=32, force_num_bin=0, cluster_ratio=5.0, inner_iter=3000, seed=2)
    prob, wl, density, ff, data = _ref_problem(nl, opts)
    n = nl.num_mov
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    pos = torch.tensor(pos0)
    args = SimpleNamespace(**vars(opts))
    stats = run_placement.global_placement_main(data, wl, density, pos, prob.node_size, ff, args, _Log())
    hpwl = float(wl.hpwl(pos))
    ovf = float(density.exact_overflow(pos[:n].contiguous()))
    np.savez_compressed(os.path.join(HERE, "golden_place2.npz"), pos0=pos0, cells=2500, nets=2620, window=80, seed=21,
                        num_bin=32, cluster_ratio=5.0, cluster_seed=2, clusters=stats["clusters"],
                        coarse_iters=stats["coarse_iters"], iters=stats["iters"], reason=stats["stop_reason"], hpwl=hpwl,
                        overflow=ovf, coarse_num_bin=stats["coarse_num_bin"])
    print("place2:", stats)


if __name__ == "__main__" and len(sys.argv) > 1:
    for name in sys.argv[1:]:
        globals()["gen_" + name]()
    sys.exit(0)

if __name__ == "__main__":
    gen_coarse()
    gen_place2()
    gen_cluster()
    gen_wa()
    gen_density()
    gen_control()
    gen_place()
    print("golden fixtures written to", HERE)
