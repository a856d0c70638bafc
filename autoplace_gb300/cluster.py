"""Two-level placement, step 1: the cells merged into clusters by rounds of star matching, on the device.

Mirrors cluster_cells (src/cluster.py:38-85) call for call: the pair edges of the small nets, then up to
`max_rounds` rounds, each with half of the clusters drawn as heads from a seeded CPU generator (torch.rand of
torch.Generator().manual_seed(seed), as the reference draws them), until the clusters are few enough or a round
merges nothing. The edge building and every round run in libgp103 (gp103_cluster_edges / _round / _relabel); the
generator's stream is drawn once per design and copied to the device, where each round compares its share with 0.5;
the host reads two counts per round. Integer weights and areas and fixed tie rules make the result
the reference's, bit for bit.
"""
import ctypes
import math
from types import SimpleNamespace

import numpy as np
import torch

from . import native


def pair_bound(pin_net, max_degree=8):
    """Number of ordered pin pairs of the nets of 2 .. max_degree pins: a bound on the pair entries."""
    deg = np.bincount(np.asarray(pin_net, np.int64))
    d = deg[(deg >= 2) & (deg <= max_degree)].astype(np.int64)
    return int((d * (d - 1)).sum())


def limits(area, ratio):
    """(big, cap) of cluster_cells, evaluated as the reference evaluates them (torch scalar arithmetic on the CPU: with
    a float ratio, cap is a float32 floor division): a cell of area >= big stays alone, two clusters merge only when
    their areas add up to at most cap (exact as integers below 2^24, the float32 range the comparison runs in)."""
    a = torch.as_tensor(np.asarray(area, np.int64))
    n = len(a)
    big = 20 * a.sum() // n
    small = a < big
    cap = 3 * ratio * a[small].sum() // (2 * int(small.sum()))
    return int(big), int(math.floor(float(cap)))


def device_limits(area_dev, ratio):
    """limits() of the cells' areas on the device (int64 [n]): the integer sums there (two host reads), the float32
    scalar arithmetic of the reference on the CPU as limits() does it -> the same (big, cap)."""
    n = int(area_dev.numel())
    if n == 0:
        return 0, 0
    big = 20 * int(area_dev.sum()) // n
    small = area_dev < big
    s, count = (int(x) for x in torch.stack([(area_dev * small).sum(), small.sum()]).cpu())
    cap = 3 * ratio * torch.tensor(s) // (2 * count)
    return int(big), int(math.floor(float(cap)))


class Stream(object):
    """The seeded CPU generator's float32 draws as one stream (torch.rand of torch.Generator().manual_seed(seed)):
    consecutive torch.rand calls on a generator give the consecutive pieces of one long draw, so the stream is drawn
    ahead in blocks, and a placement's rounds take the next `num` values each -- the numbers the reference's calls
    give. Every placement with this seed reads the same stream from its start; the drawn part is kept."""

    def __init__(self, seed, block):
        self.gen = torch.Generator().manual_seed(int(seed))
        self.block = max(int(block), 1)
        self.buf = np.zeros(0, np.float32)

    def upto(self, count):
        while len(self.buf) < count:
            more = max(self.block, count - len(self.buf))
            self.buf = np.concatenate([self.buf, torch.rand(more, generator=self.gen).numpy()])
        return self.buf


def seeded_uniform(seed, count, device="cuda", stream=None):
    """torch.rand(count, generator=torch.Generator().manual_seed(seed)) (the CPU generator's stream, the same bits)
    made on the device (gp103_seeded_uniform). -> float32 device tensor [count]."""
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    with torch.cuda.stream(stream):
        out = torch.empty(max(int(count), 1), dtype=torch.float32, device=dev)
    native.call("gp103_seeded_uniform", int(seed), int(count), ctypes.c_void_p(out.data_ptr()), stream.cuda_stream)
    return out[:int(count)]


def device_pair_bound(pin_net, num_nets, max_degree=8):
    """pair_bound of the pins' nets already on the device (int32 [P]), one host read."""
    deg = torch.bincount(pin_net.long(), minlength=max(int(num_nets), 1))
    d = deg[(deg >= 2) & (deg <= max_degree)]
    return int((d * (d - 1)).sum())


def prepare(prob, device="cuda", stream=None, max_degree=8, draw_stream=None):
    """What a placement's clustering needs of its design, made once per design (like the cells' own uploads): the
    pins on the device (int32 cells and nets, float32 offsets: the device problem's own, else uploaded), the cells'
    areas and the merge limits, the pair bound, the heads' seeded stream drawn ahead (four draws per cell) and
    expand's seeded draws. -> SimpleNamespace."""
    nl, o, n = prob.nl, prob.opts, prob.num_mov
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    with torch.cuda.stream(stream):
        if torch.is_tensor(getattr(prob, "all_net", None)) and prob.all_net.is_cuda:
            pc, pn, po = prob.all_cell, prob.all_net, prob.all_off
        else:
            pc = torch.as_tensor(np.asarray(nl.pin_cell, np.int32)).to(dev, non_blocking=True)
            pn = torch.as_tensor(np.asarray(nl.pin_net, np.int32)).to(dev, non_blocking=True)
            po = torch.as_tensor(np.asarray(nl.pin_off, np.float32)).to(dev, non_blocking=True)
        bound = device_pair_bound(pn, nl.num_nets, max_degree)
    # the seeded draws, made on the device: the heads' stream (six per cell; the 12 rounds of the 1.2M-cell netlist
    # read 4.07 per cell; a longer need extends it from the host's generator) and expand's draws, which are the same
    # stream's start (the reference seeds expand's generator with the same seed: its first 2 n values)
    heads = Stream(o.seed, n)
    # (on draw_stream when given: the draws, ~2 ms in one block, then run beside the caller's set-up on `stream`;
    # coarse_problem waits for them before the first round)
    heads_dev = seeded_uniform(o.seed, 6 * n, dev, draw_stream or stream)
    ready = None
    if draw_stream is not None:
        ready = torch.cuda.Event()
        ready.record(draw_stream)
    with torch.cuda.stream(stream):
        on_dev = getattr(prob, "node_size_dev", None)
        if torch.is_tensor(on_dev) and on_dev.device == dev:
            size_dev = on_dev[:n].float()
        else:
            size_dev = torch.as_tensor(np.asarray(prob.node_size[:n], np.float32)).to(dev, non_blocking=True)
        # the areas in 1/1024 of a site area, rounded from the float32 area (the reference's, bit for bit: float32
        # products, then exact float64 scaling and half-to-even rounding)
        area_dev = torch.round((size_dev[:, 0] * size_dev[:, 1]).double() * 1024).long()
        lim = device_limits(area_dev, o.cluster_ratio)
    return SimpleNamespace(pins=(pc, pn), pin_off=po, area=None, area_dev=area_dev, size_dev=size_dev,
                           limits=lim, pair_bound=max(bound, 1),
                           num_nets=int(nl.num_nets), seed=int(o.seed), heads=heads, heads_dev=heads_dev,
                           expand_draws=heads_dev[:2 * n].view(n, 2), draws_ready=ready)


def cluster_cells(pin_cell, pin_net, area, ratio, seed, max_degree=8, per_head=3, max_rounds=12, device="cuda",
                  draws=None, stream=None, dev_pins=None, prep=None, on_device=False):
    """pin_cell / pin_net [P] sorted by net (cell index len(area) = a fixed pin); area [n] int64. -> (cluster of
    every cell [n] int64, area of every cluster [K] int64), as numpy arrays. draws(round, num) -> float32 [num] can
    stand in for the seeded generator (tests). dev_pins: (pin_cell, pin_net) already on the device as int32. prep:
    prepare()'s result for this design (pins, limits, pair bound, the seeded stream), made once per design.
    on_device: -> (cluster of every cell [n] int32, area of every cluster [K] int64) as device tensors instead."""
    if prep is not None:                        # (the areas and limits on the device)
        n = int(prep.area_dev.numel())
    else:
        area = np.ascontiguousarray(area, np.int64)
        n = len(area)
    if n == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    if prep is not None:
        (big, cap), num_nets, E, dev_pins = prep.limits, prep.num_nets, prep.pair_bound, prep.pins
        npins = int(prep.pins[0].shape[0])
    else:
        big, cap = limits(area, ratio)
        pin_net = np.asarray(pin_net, np.int64)
        num_nets = int(pin_net.max()) + 1 if len(pin_net) else 0
        E = max(pair_bound(pin_net, max_degree), 1)
        npins = len(pin_net)
    with torch.cuda.stream(stream):
        if dev_pins is not None:
            pc, pn = dev_pins
        else:
            pc = torch.as_tensor(np.asarray(pin_cell, np.int32)).to(dev)
            pn = torch.as_tensor(np.asarray(pin_net, np.int32)).to(dev)
        scratch = torch.empty(int(native.lib().gp103_cluster_scratch(n, num_nets, E)), dtype=torch.uint8, device=dev)
        rows = [torch.zeros(n + 1, dtype=torch.int32, device=dev) for _ in range(2)]
        col = [torch.zeros(E, dtype=torch.int32, device=dev) for _ in range(2)]
        wgt = [torch.zeros(E, dtype=torch.int32, device=dev) for _ in range(2)]
        areas = [prep.area_dev.clone() if prep is not None else torch.as_tensor(area).to(dev),
                 torch.zeros(n, dtype=torch.int64, device=dev)]
        counts = torch.zeros(2, dtype=torch.int32, device=dev)
        new_index = torch.zeros(n, dtype=torch.int32, device=dev)
        cid = torch.arange(n, dtype=torch.int32, device=dev)
    native.call("gp103_cluster_edges", p(pc), p(pn), npins, num_nets, n, max_degree, E, p(scratch),
                scratch.numel(), p(rows[0]), p(col[0]), p(wgt[0]), p(counts), s)
    stream.synchronize()
    if int(counts[1]) > E:
        raise RuntimeError("pair bound too small: %d > %d" % (int(counts[1]), E))
    heads = prep.heads if prep is not None else Stream(seed, n)
    drawn = prep.heads_dev if prep is not None and draws is None else None   # the stream's start, on the device
    num, a, at = n, 0, 0
    for r in range(max_rounds):
        if num * ratio <= n:
            break
        if drawn is not None and at + num > drawn.numel():          # the stream's next part, on the device once
            buf = heads.upto(at + num)
            with torch.cuda.stream(stream):
                drawn = torch.cat([drawn, torch.as_tensor(buf[drawn.numel():]).to(dev)])
            prep.heads_dev = drawn
        if drawn is not None:
            with torch.cuda.stream(stream):
                head = (drawn[at:at + num] < 0.5).to(torch.uint8)
        else:
            d = draws(r, num) if draws is not None else heads.upto(at + num)[at:at + num]
            head = torch.as_tensor(np.asarray(d) < np.float32(0.5)).to(torch.uint8)
            with torch.cuda.stream(stream):
                head = head.to(dev)
        at += num
        b = 1 - a
        native.call("gp103_cluster_round", p(rows[a]), p(col[a]), p(wgt[a]), num, E, p(areas[a]), p(head),
                    cap, big, per_head, p(scratch), scratch.numel(), p(new_index), p(areas[b]), p(rows[b]), p(col[b]),
                    p(wgt[b]), p(counts), s)
        stream.synchronize()
        kept = int(counts[0])
        if kept == num:
            break
        native.call("gp103_cluster_relabel", p(cid), n, p(new_index), s)
        num, a = kept, b
    if on_device:
        return cid, areas[a][:num]
    stream.synchronize()
    return cid.cpu().numpy().astype(np.int64), areas[a][:num].cpu().numpy()


class Clusters(object):
    """coarse_problem's result: cid_dev [n] (device int32), num, size [num, 2] float32 (host), single_dev [num]
    (device uint8), problem, prep; cid [n] (host int64) downloaded on first use."""

    def __init__(self, cid_dev, num, size, single_dev, problem, prep):
        self.cid_dev, self.num, self.size, self.single_dev = cid_dev, num, size, single_dev
        self.problem, self.prep, self._cid = problem, prep, None

    @property
    def cid(self):
        if self._cid is None:
            self._cid = self.cid_dev.cpu().numpy().astype(np.int64)
        return self._cid


def coarse_problem(prob, device="cuda", stream=None, build="device", prep=None):
    """The problem of the clusters (coarse_problem, src/cluster.py:88-130), from a cell-level Problem:
      - the cells clustered (cluster_cells, areas in 1/1024 of a site area, rounded from the float32 area);
      - a merged cluster is a square of its summed area with its pins at the centre, one per net; a cluster of one
        cell keeps its shape and pins (the pin selection runs on the device: gp103_coarse_pins);
      - the same fillers, target and options; one grid, between the overflow grid and the cells' force grid, as
        the cells' grid follows the cells.
    build: "device" = the clusters' per-pin and per-node arrays built on the device from the selected pins
    (Problem.on_device: torch tensors), "host" = downloaded and built in numpy (the same arrays, bit for bit).
    prep: prepare(prob)'s result (the design's pins on the device, areas, limits, seeded draws), made once per design.
    -> SimpleNamespace(cid [n], num, size [num, 2] float32, problem: the clusters' Problem, prep)."""
    from . import problem as P
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    nl, o, n = prob.nl, prob.opts, prob.num_mov
    P_ = len(nl.pin_cell)
    if prep is None:
        prep = prepare(prob, device=dev, stream=stream)
    (pc, pn), po, area = prep.pins, prep.pin_off, prep.area
    if getattr(prep, "draws_ready", None) is not None:
        stream.wait_event(prep.draws_ready)         # the seeded draws, made on another stream
        prep.draws_ready = None
    cd, carea = cluster_cells(nl.pin_cell, nl.pin_net, area, o.cluster_ratio, o.seed, device=device, stream=stream,
                              prep=prep, on_device=True)
    num = int(carea.shape[0])
    # sizes: a merged cluster the square of its summed area, a one-cell cluster its cell's (gp103_cluster_members)
    with torch.cuda.stream(stream):
        cnt_c = torch.empty(max(num, 1), dtype=torch.int32, device=dev)
        sg = torch.empty(max(num, 1), dtype=torch.uint8, device=dev)
        csize_dev = torch.empty((max(num, 1), 2), dtype=torch.float32, device=dev)
    native.call("gp103_cluster_members", p(cd), n, num, p(carea), p(prep.size_dev), p(cnt_c), p(sg), p(csize_dev), s)
    csize = csize_dev[:num].cpu().numpy()
    # pins: on the device
    with torch.cuda.stream(stream):
        scratch = torch.empty(int(native.lib().gp103_coarse_pins_scratch(P_)), dtype=torch.uint8, device=dev)
        oc = torch.empty(max(P_, 1), dtype=torch.int32, device=dev)
        oo = torch.empty((max(P_, 1), 2), dtype=torch.float32, device=dev)
        on = torch.empty(max(P_, 1), dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    native.call("gp103_coarse_pins", p(pc), p(po), p(pn), P_, n, p(cd), num, p(sg), p(scratch), scratch.numel(),
                p(oc), p(oo), p(on), p(cnt), s)
    stream.synchronize()
    k = int(cnt.item())
    # the grid: as the cells' force grid follows the cells (at most the cells' grid)
    fine_ff = getattr(prob, "fixed_fraction", None)
    if fine_ff is None:
        fine_ff = nl.fixed_fraction(prob.force_bin, prob.force_bin)
    nb = min(prob.force_bin, P.force_num_bin(num, 1.0 - float(fine_ff.mean()), prob.num_bin))
    if nb == prob.force_bin:
        fixed_fraction = fine_ff
    elif nb == prob.num_bin and getattr(prob, "judge_fraction", None) is not None:
        fixed_fraction = prob.judge_fraction
    else:
        fixed_fraction = device_fixed_fraction(nl, nb, nb, device=dev, stream=stream)
    copts = SimpleNamespace(**vars(o))
    copts.settle_iter, copts.min_iter = 0, 0
    if build == "host":
        c_cell, c_off, c_net = oc[:k].cpu().numpy(), oo[:k].cpu().numpy(), on[:k].cpu().numpy()
        cprob = P.Problem.clusters(prob, csize, c_cell, c_off, c_net, nb, fixed_fraction, copts)
    else:
        pins = dict(pin_cell=oc[:k], pin_off=oo[:k], pin_net=on[:k])
        cprob = P.Problem.clusters(prob, csize, pins["pin_cell"], pins["pin_off"], pins["pin_net"], nb,
                                   fixed_fraction, copts, arrays=False)
        pins["node_size"] = np.ascontiguousarray(cprob.node_size, np.float64)
        cprob = cprob.on_device(dev, stream, host=pins)
    return Clusters(cd, num, csize, sg[:num], cprob, prep)


def device_fixed_fraction(nl, nbx, nby, device="cuda", stream=None):
    """nl.fixed_fraction(nbx, nby) computed on the device (gp103_macro_fraction: the same bits) -> float64 numpy
    [nbx, nby]."""
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    rects = np.ascontiguousarray(np.asarray(nl.macros, np.float64).reshape(-1, 4))
    with torch.cuda.stream(stream):
        r = torch.as_tensor(rects).to(dev) if len(rects) else None
        out = torch.empty((nbx, nby), dtype=torch.float64, device=dev)
    native.call("gp103_macro_fraction", None if r is None else ctypes.c_void_p(r.data_ptr()), len(rects),
                float(nl.width), float(nl.height), nbx, nby, ctypes.c_void_p(out.data_ptr()), stream.cuda_stream)
    return out.cpu().numpy()


def expand(cpos, coarse, prob, seed, device="cuda", stream=None):
    """Positions of clusters + fillers ([num + F, 2], host or device) -> positions of cells + fillers (expand,
    src/cluster.py:133-144): a cell at a random point of its cluster's square, the draws from the seeded CPU
    generator as the reference takes them; the fillers keep theirs. -> device tensor [n + F, 2]."""
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    n, num = prob.num_mov, coarse.num
    prep = getattr(coarse, "prep", None)
    if prep is not None and prep.seed == int(seed):
        r = prep.expand_draws                           # (the seeded draws, made once per design)
    else:
        gen = torch.Generator().manual_seed(int(seed))
        r = torch.rand(n, 2, generator=gen)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    with torch.cuda.stream(stream):
        cpos = torch.as_tensor(cpos, dtype=torch.float32).to(dev).contiguous()
        out = torch.empty((n + cpos.shape[0] - num, 2), dtype=torch.float32, device=dev)
        out[n:] = cpos[num:]
        cid = coarse.cid_dev if hasattr(coarse, "cid_dev") else torch.as_tensor(coarse.cid.astype(np.int32)).to(dev)
        cs = torch.as_tensor(coarse.size).to(dev)
        sz = torch.as_tensor(np.asarray(prob.node_size[:n], np.float32)).to(dev)
        rd = r.to(dev)
    native.call("gp103_expand", p(cpos), p(cid), p(cs), p(sz), p(rd), n, p(out), stream.cuda_stream)
    stream.synchronize()
    return out
