"""The placement loop on the GPU: one level of AutoPlace's global placement run by libgp103's fused passes.

Mirrors `_place_level` + `run_level_on_gpu` (src/run_placement.py:41-76, src/gpu_loop.py:35-81):
  1. first step length from a probe step (estimate_initial_learning_rate, src/nesterov_optimizer.py:56-61) and the
     optimiser's own probe (NesterovOptimizer.__init__, :15-32): four gradient evaluations, four scalars read back;
  2. the wirelength-only start (density weight 0) until the WA wirelength settles (ParamScheduler.start_step),
     control on the device, the host polling every `check_every` passes;
  3. the first density weight in tension units (Objective.tension_unit, src/calculator.py:20-24);
  4. the density phase: `check_every` passes per CUDA-graph replay until the control kernel stops the run.
Device buffers come from torch's caching allocator (plumbing only); every kernel is libgp103's, launched on one
stream. A pass runs on the positions in the ping-pong buffers selected by a device index, so the passes of a
graph never need the host.
"""
import ctypes
import math
import time

import numpy as np
import torch

from . import native
from .native import Plan, Sizes, T as TI, T_SIZE

S_FIELDS = ("lam gam alpha a iter hpwl_prev motion ww mu settled best_hpwl best_ovf is_best improved stop accept "
            "loop_it evals res_hpwl res_ovf has_best").split()
SK = {n: i for i, n in enumerate(S_FIELDS)}
REASON = {1: "converged", 2: "stalled", 3: "diverged", 4: "max_iter", 5: "handover", 6: "device_error"}
STOP_DEVICE_ERROR = 6


START_EVERY = 4        # passes per poll of the wirelength-only start
_GRAPH_LAUNCHES = {"captured": 0, "replayed": 0}        # libgp103 launches inside CUDA graphs, all Placers
SHORT_NET = 8          # nets of up to this many pins are done one per thread (WA_REG of the kernel)
MID_NET = 16           # nets of up to this many pins (and more than SHORT_NET) are done by 4 lanes each
G8_NET = 32            # ... by 8 lanes each (nets of MID_NET + 1 .. G8_NET pins)
G16_NET = 64           # ... by 16 lanes each (G8_NET + 1 .. G16_NET pins); longer nets by a warp each


def net_order(net_start, cell32, cell_pin):
    """The device order of the optimised nets: short nets (<= SHORT_NET pins) first, in classes of 2, 3 and 4..8
    pins so that a warp's lanes do equal work, each class ordered by the net's lowest cell (nearby nets gather
    nearby cells); the long nets after them in classes of 9..16, 17..32, 33..64 pins (groups of 4, 8, 16 lanes) and
    longer (a warp each). Pins move with their nets.
    -> (pin permutation: new position -> old pin, new net_start, slot: new pin position -> its position in cell
    order (cell_pin order, which every cell sums in), then the class boundaries as gp103_net_order's split: the
    numbers of nets of up to SHORT_NET, MID_NET, 2, 3, G8_NET and G16_NET pins)."""
    ns = np.asarray(net_start, np.int64)
    deg = np.diff(ns)
    n = len(deg)
    if n == 0:
        return np.zeros(0, np.int64), np.zeros(1, np.int32), np.zeros(0, np.int32), 0, 0, 0, 0, 0, 0
    first = np.minimum.reduceat(np.asarray(cell32, np.int64), ns[:-1]) if len(cell32) else np.zeros(n, np.int64)
    cls = np.select([deg == 2, deg == 3, deg <= SHORT_NET, deg <= MID_NET, deg <= G8_NET, deg <= G16_NET],
                    [0, 1, 2, 3, 4, 5], 6)
    order = np.lexsort((first, cls))
    lens = deg[order]
    new_start = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    perm = np.repeat(ns[:-1][order] - new_start[:-1], lens) + np.arange(int(new_start[-1]))
    newpos = np.empty_like(perm)
    newpos[perm] = np.arange(len(perm))
    slot = np.empty(len(perm), np.int64)
    slot[newpos[np.asarray(cell_pin, np.int64)]] = np.arange(len(perm))
    return (perm, new_start.astype(np.int32), slot.astype(np.int32), int((cls < 3).sum()), int((cls < 4).sum()),
            int((cls < 1).sum()), int((cls < 2).sum()), int((cls < 5).sum()), int((cls < 6).sum()))


def launches():
    """Kernels of libgp103 executed so far by this process, every Placer's graph replays counted launch by launch
    (a captured launch counts when its graph replays, not when it is captured)."""
    return native.launch_count() - _GRAPH_LAUNCHES["captured"] + _GRAPH_LAUNCHES["replayed"]


def wa_long_share(num_pins, first_long_pin):
    """The share (percent) of the fused WA launch's blocks given to the long nets (9 pins or more), from the share f
    of the pins they hold: 30 + 60 f, within 40 .. 75. Measured best shares: 50-55 on the 1.2M-cell netlist
    (f = 0.38: 53 here), 60-65 on its clusters (f = 0.53: 62)."""
    if num_pins <= 0:
        return 0
    f = (num_pins - first_long_pin) / float(num_pins)
    return int(min(75, max(40, round(30 + 60 * f))))


def side_stream(stream):
    """A stream other than `stream` for the WA kernels of split passes. torch hands out its streams from a small
    pool, round robin, so a new torch.cuda.Stream can be `stream` itself: draw until it is not."""
    for _ in range(64):
        s = torch.cuda.Stream(stream.device)
        if s.cuda_stream != stream.cuda_stream:
            return s
    raise RuntimeError("no CUDA stream other than the pass's own")


def field_mode(mode, nbx, nby):
    """The field mode a grid of nbx x nby bins runs in: `mode`, or fp32 where the tensor-core field cannot tile the
    grid (gp103_plan_sizes answers GP103_ERR_SHAPE)."""
    if mode == native.FIELD_FP32:
        return mode
    rc = native.lib().gp103_plan_sizes(nbx, nby, mode, ctypes.byref(Sizes()))
    if rc == native.ERR_SHAPE:
        return native.FIELD_FP32
    native.check(rc, "gp103_plan_sizes")
    return mode


def mean_density(prob):
    """The force grid's mean density: the nodes' area over the bin area plus the fixed map, over the bins. Every node
    stays inside the region (positions are clamped), so this is the mean of every pass's density map; it is the
    field's shift (gp103_plan.field_shift)."""
    f = prob.force
    area = prob.area
    total = float(area.double().sum()) if torch.is_tensor(area) else float(np.asarray(area, np.float64).sum())
    fixed = float(np.asarray(f.fixed_map, np.float64).sum())
    return (total / f.bin_area + fixed) / (f.nbx * f.nby)


def _tensor(a, dt):
    """A host array or a tensor (host or device, e.g. from Problem.on_device) as a tensor of type dt."""
    if torch.is_tensor(a):
        return a.to(dtype=dt)
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt)


def pinned_inputs(prob):
    """The problem arrays a Placer uploads, as pinned CPU tensors ({name: tensor}). A caller that keeps its inputs in
    pinned memory passes them as Placer(prob, host=...): the uploads are then asynchronous DMA copies."""
    cs, f, j = prob.csr, prob.force, prob.judge
    arrays = dict(net_start=cs.net_start, cell32=cs.cell32, off=cs.off, cell_pin=cs.cell_pin, cell_start=cs.cell_start,
                  size=f.size, ratio=f.ratio, pins=prob.pins, area=prob.area, lo=f.pos_lo, hi=f.pos_hi,
                  fixed=f.fixed_map)
    if j is not None:
        arrays.update(jsize=j.size, jratio=j.ratio, jfixed=j.fixed_map)
    return {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in arrays.items()}


class Placer(object):
    def __init__(self, prob, field="f16x3", device=None, check_every=16, use_graphs=True, stream=None,
                 sort_every=None, host=None, handover_gamma=0.0, split=False, side=None):
        """host: optional {name: pinned CPU tensor} holding the problem's arrays (pinned_inputs), uploaded instead
        of the Problem's numpy arrays. handover_gamma: a run on clusters stops ("handover") once its smoothing is
        down to this (the smoothing the cells start with); 0 = never.
        A tensor-core field (f16x3, bf16x6, bf16x3) needs a grid of multiples of 128 bins per side: on a smaller grid
        (clusters, small designs) the field runs in fp32.
        split: density passes with the WA kernels on a second stream (`side`, or one drawn by side_stream), beside
        the density map and the field (gp103_pass_split); the same results. Off for a Placer of its own; Flow turns
        it on for both levels (at the 1.2M-cell netlist: the clusters' level 38.2 -> 35.5 ms, the cells' 46.3 ->
        44.9 ms). split="field": the passes wait for the WA kernels before the field instead of before the gather
        (GP103_PASS_JOIN_FIELD; the same time at the 1.2M-cell netlist)."""
        self.p = prob
        self.dev = torch.device(device or "cuda")
        self.mode = field_mode(native.FIELD_MODES[field] if isinstance(field, str) else int(field),
                               prob.force.nbx, prob.force.nby)
        self.handover_gamma = float(handover_gamma or 0.0)
        self.start_gamma = 10 * prob.base_gamma     # the WA smoothing of a fresh run (src/param_scheduler.py:31)
        self.check_every = check_every
        self.use_graphs = use_graphs
        # density passes between refreshes of the scatter's spatial order (an order only speeds the scatter up)
        self.sort_every = max(int(sort_every or check_every), 1)
        self.stream = stream or torch.cuda.Stream(self.dev)
        self.split = bool(split)
        # where the passes wait for the WA kernels of the side stream: before the gather (split=True) or before the
        # field (split="field": the WA kernels share the GPU with the density map only)
        self.split_join = "field" if split == "field" else "gather"
        self.side = (side or side_stream(self.stream)) if self.split else None
        if self.side is not None and self.side.cuda_stream == self.stream.cuda_stream:
            raise ValueError("the side stream of a split pass must differ from the pass's stream")
        self._events = []
        if self.split:
            for _ in range(2):
                e = ctypes.c_void_p()
                native.call("gp103_event_create", ctypes.byref(e))
                self._events.append(e)
        self._graphs = {}
        self._captured = self._replayed = 0
        self._keep = []
        with torch.cuda.stream(self.stream):       # every upload and set-up kernel in the stream of the passes
            self._setup(prob, host or {})

    def _setup(self, prob, host):
        dev = self.dev
        up = lambda name, a, dt: _tensor(host[name] if name in host else a, dt).to(dev, non_blocking=True)
        t = lambda a, dt: self._hold(_tensor(a, dt).to(dev, non_blocking=True))
        z = lambda shape, dt: self._hold(torch.zeros(shape, dtype=dt, device=dev))
        cs = prob.csr
        n, f, judge = prob.num_nodes, prob.force, prob.judge
        P, N = len(cs.cell32), cs.num_nets
        sz = Sizes()
        native.call("gp103_plan_sizes", f.nbx, f.nby, self.mode, ctypes.byref(sz))
        pl = Plan()
        pl.num_nodes, pl.num_mov, pl.num_nets, pl.num_pins = n, prob.num_mov, N, P
        pl.nbx, pl.nby = f.nbx, f.nby
        pl.field_mode = self.mode
        # the optimised pin set as built, reordered on the device for the WA kernels (gp103_net_order)
        ns_in, cell_in = up("net_start", cs.net_start, torch.int32), up("cell32", cs.cell32, torch.int32)
        off_in, cp_in = up("off", cs.off, torch.float32), up("cell_pin", cs.cell_pin, torch.int32)
        self.cell_start = self._hold(up("cell_start", cs.cell_start, torch.int32))
        self.pin_cell, self.pin_off = z((max(P, 1),), torch.int32), z((max(P, 1), 2), torch.float32)
        self.net_start, self.pin_slot = z((N + 1,), torch.int32), z((max(P, 1),), torch.int32)
        split = torch.zeros(6, dtype=torch.int32, device=dev)
        scratch = torch.empty(int(native.lib().gp103_net_order_scratch(N, P, prob.num_mov)), dtype=torch.uint8,
                              device=dev)
        native.call("gp103_net_order", self._p(ns_in), self._p(cell_in), self._p(off_in), self._p(cp_in), N, P,
                    prob.num_mov, self._p(scratch), scratch.numel(), self._p(self.net_start), self._p(self.pin_cell),
                    self._p(self.pin_off), self._p(self.pin_slot), self._p(split), self.stream.cuda_stream)
        pl.pin_cell, pl.pin_off, pl.net_start = self._p(self.pin_cell), self._p(self.pin_off), self._p(self.net_start)
        # the pin gradients stay in net order (the WA kernels' stores are contiguous); the gather reads each cell's
        # pins, in cell_pin order, through cell_pin_net = the inverse of pin_slot (the same sums, bit for bit; on the
        # 1.2M-cell pass 0.284 ms against 0.288 ms with the gradients stored in cell order)
        with torch.cuda.stream(self.stream):
            self.cell_pin_net = self._hold(torch.empty(max(P, 1), dtype=torch.int32, device=dev))
            if P:
                self.cell_pin_net[self.pin_slot[:P].long()] = torch.arange(P, dtype=torch.int32, device=dev)
        pl.cell_start, pl.cell_pin, pl.pin_slot = self._p(self.cell_start), self._p(self.cell_pin_net), None
        # (the stream-ordered allocator may hand these blocks to the allocations below: their kernels run after
        # gp103_net_order on the same stream; the split counts are read back at the end, after the other set-up)
        del ns_in, cell_in, off_in, cp_in, scratch
        self.size = self._hold(up("size", f.size, torch.float32))
        self.ratio = self._hold(up("ratio", f.ratio, torch.float32))
        self.pins = self._hold(up("pins", prob.pins, torch.float32))
        self.area = self._hold(up("area", prob.area, torch.float32))
        self.lo = self._hold(up("lo", f.pos_lo, torch.float32))
        self.hi = self._hold(up("hi", f.pos_hi, torch.float32))
        for k in ("size", "ratio", "pins", "area", "lo", "hi"):
            setattr(pl, k, self._p(getattr(self, k)))
        pl.bx, pl.by, pl.target = f.bx, f.by, prob.target
        pl.field_shift = mean_density(prob)
        self.fixed = self._hold(up("fixed", f.fixed_map, torch.float32))
        pl.fixed = self._p(self.fixed)
        pl.ovf_scale = f.bin_area / f.mov_area
        if judge is not None:
            pl.jnbx, pl.jnby = judge.nbx, judge.nby
            self.jsize = self._hold(up("jsize", judge.size, torch.float32))
            self.jratio = self._hold(up("jratio", judge.ratio, torch.float32))
            self.jfixed = self._hold(up("jfixed", judge.fixed_map, torch.float32))
            pl.jsize, pl.jratio, pl.jfixed = self._p(self.jsize), self._p(self.jratio), self._p(self.jfixed)
            pl.jbx, pl.jby = judge.bx, judge.by
            pl.jovf_scale = judge.bin_area / judge.mov_area
            self.jmap = z((judge.nbx, judge.nby), torch.int64)
            pl.jmap = self._p(self.jmap)
        self.field_const = z((sz.field_const,), torch.uint8)
        self.field_work = z((sz.field_work,), torch.uint8)
        self.ex, self.ey = z((f.nbx, f.nby), torch.float32), z((f.nbx, f.nby), torch.float32)
        pl.field_const, pl.field_work, pl.ex, pl.ey = (self._p(x) for x in (self.field_const, self.field_work,
                                                                             self.ex, self.ey))
        self.U = [z((n, 2), torch.float32) for _ in range(2)]
        self.V = [z((n, 2), torch.float32) for _ in range(2)]
        self.G = [z((n, 2), torch.float32) for _ in range(2)]
        for k in range(2):
            pl.u[k], pl.v[k], pl.g[k] = self._p(self.U[k]), self._p(self.V[k]), self._p(self.G[k])
        self.best = z((n, 2), torch.float32)
        # pinned host copies of the state (two, alternating) and their events, for the host's polls
        self._s_host = [(torch.zeros(len(S_FIELDS), dtype=torch.float64).pin_memory(), torch.cuda.Event())
                        for _ in range(2)]
        self.cur = z((1,), torch.int32)
        self.S = z((len(S_FIELDS),), torch.float64)
        self.T = z((T_SIZE,), torch.float64)
        self.kp = z((5,), torch.float32)
        self.c = t(prob.constants(self.handover_gamma), torch.float64)
        self.pin_grad = z((max(P, 1), 2), torch.float32)
        self.map = z((2, f.nbx, f.nby), torch.int64)
        self.red = z((sz.red,), torch.float64)
        self.counters = z((16,), torch.int32)
        self.scal = z((8,), torch.float64)
        self.order = self._hold(torch.arange(n, dtype=torch.int32, device=dev))
        self.order_counts = z((2048,), torch.int32)
        self.order_cursor = z((2048,), torch.int32)
        pl.order, pl.order_counts, pl.order_cursor = (self._p(x) for x in (self.order, self.order_counts,
                                                                            self.order_cursor))
        self.tmp = [z((n, 2), torch.float32) for _ in range(2)]
        for k in ("best", "cur", "S", "T", "kp", "c", "pin_grad", "map", "red", "counters"):
            setattr(pl, k, self._p(getattr(self, k)))
        native.call("gp103_field_constants", ctypes.byref(pl), self.stream.cuda_stream)
        # the one host synchronisation of the set-up: the net classes of the WA order (launch sizes of the passes)
        # and the first pin of the long nets (gathered on the device)
        with torch.cuda.stream(self.stream):
            first_long = self.net_start[split[0].long()].view(1)
        (pl.net_split, pl.net_mid, pl.net_two, pl.net_three, self.net_g8, self.net_g16,
         first_long) = (int(x) for x in torch.cat([split, first_long]).cpu().tolist())
        # the default partition of the long nets: 9-16 pins by 4 lanes, longer ones a warp each (the 8- and 16-lane
        # groups of 17-32 and 33-64 pins are an autotuner choice: tune.apply_wa)
        pl.net_g8 = pl.net_g16 = 0
        pl.wa_long_share = wa_long_share(P, first_long)
        self.plan = pl
        self._ref = ctypes.byref(pl)

    def __del__(self):
        try:
            for e in getattr(self, "_events", []):
                native.lib().gp103_event_destroy(e)
        except Exception:
            pass

    # ------------------------------------------------------------------ helpers
    def _hold(self, x):
        self._keep.append(x)
        return x

    @staticmethod
    def _p(x):
        return ctypes.c_void_p(x.data_ptr())

    def sync(self):
        self.stream.synchronize()

    def check_device(self, what="gp103"):
        """Raise RuntimeError if a wait of the tensor-core field ran out (the plan's device error flag), after the
        work queued so far. The flag stays set: a later run stops at once with reason device_error."""
        code = native.device_error(self._ref, self.stream.cuda_stream)
        if code:
            native.raise_device_error(code, what)

    def clear_device_error(self):
        """Reset the device error flag (after a failure was handled), -> the code it held."""
        return native.device_error(self._ref, self.stream.cuda_stream, clear=True)

    def eval(self, pos, g_out, g_ref=None, weight=0.0, precond=-1.0, with_wl=True):
        """-> (|g - g_ref|^2, WA, HPWL, overflow sum, L1 of g over the cells), after a host sync."""
        native.call("gp103_eval", self._ref, self._p(pos), self._p(g_out),
                    None if g_ref is None else self._p(g_ref), float(weight), float(precond), int(bool(with_wl)),
                    self._p(self.scal), self.stream.cuda_stream)
        if weight != 0.0:
            self.check_device("gp103_eval")                  # (synchronises the stream)
        self.sync()
        return self.scal[:5].cpu().numpy()

    def probe(self, v, g, step, out):
        native.call("gp103_probe", self._ref, self._p(v), self._p(g), float(step), self._p(out), self._p(self.scal),
                    self.stream.cuda_stream)
        self.sync()
        return float(self.scal[0].cpu())

    def _passes(self, phase, k, split=None, sort=True):
        s = self.stream.cuda_stream
        split = self.split if split is None else split
        for i in range(k):
            sort_now = sort and phase == native.PHASE_DENSITY and i % self.sort_every == 0
            flags = phase | (native.PASS_SORT if sort_now else 0)
            if split and phase == native.PHASE_DENSITY:
                if self.split_join == "field":
                    flags |= native.PASS_JOIN_FIELD
                native.call("gp103_pass_split", self._ref, flags, s, self.side.cuda_stream, self._events[0],
                            self._events[1])
            else:
                native.call("gp103_pass", self._ref, flags, s)

    def _replay(self, phase):
        # the wirelength-only start ends after ~10 passes: it polls every START_EVERY passes, the density phase every
        # check_every
        k = self.check_every if phase == native.PHASE_DENSITY else min(START_EVERY, self.check_every)
        if not self.use_graphs:
            self._passes(phase, k)
            return
        g = self._graphs.get(phase)
        if g is None:
            g = torch.cuda.CUDAGraph()
            before = native.launch_count()
            with torch.cuda.graph(g, stream=self.stream):
                self._passes(phase, k)
            per = native.launch_count() - before
            self._captured += per
            _GRAPH_LAUNCHES["captured"] += per
            self._graphs[phase] = (g, per)
        g, per = self._graphs[phase]
        with torch.cuda.stream(self.stream):
            g.replay()
        self._replayed += per
        _GRAPH_LAUNCHES["replayed"] += per

    def launches(self):
        """Kernels of libgp103 executed so far by this process (graph replays counted launch by launch)."""
        return launches()

    def overflow_scale(self):
        return self.plan.jovf_scale if self.plan.jnbx > 0 else self.plan.ovf_scale

    def evaluate(self, pos):
        """The judges of a placement, in float64 on the device: (HPWL over every net, overflow of the movable cells
        with their real sizes on the overflow grid). The whole netlist is uploaded on the first call."""
        p = self.p
        if not hasattr(self, "_ev"):
            t = lambda a, dt: _tensor(a, dt).to(self.dev, non_blocking=True)
            gr = p.real_judge
            with torch.cuda.stream(self.stream):
                self._ev = dict(cell=t(p.all_cell, torch.int32), off=t(p.all_off, torch.float32),
                                start=t(p.all_net_start, torch.int32), size=t(p.nl.size, torch.float32),
                                fixed=t(gr.fixed_map, torch.float32),
                                map=torch.zeros((gr.nbx, gr.nby), dtype=torch.int64, device=self.dev),
                                scratch=torch.zeros(native.EVAL_SCRATCH_BYTES, dtype=torch.uint8, device=self.dev),
                                out=torch.zeros(2, dtype=torch.float64, device=self.dev), grid=gr)
        e, gr, s = self._ev, self._ev["grid"], self.stream.cuda_stream
        with torch.cuda.stream(self.stream):
            pos = torch.as_tensor(pos, dtype=torch.float32).to(self.dev).contiguous()
        out = e["out"]
        native.call("gp103_hpwl", self._p(pos), self._p(e["cell"]), self._p(e["off"]), self._p(e["start"]),
                    len(p.all_net_start) - 1, p.num_mov, self._p(e["scratch"]), ctypes.c_void_p(out.data_ptr()), s)
        native.call("gp103_exact_overflow", self._p(pos), self._p(e["size"]), p.num_mov, gr.bx, gr.by, gr.nbx,
                    gr.nby, self._p(e["fixed"]), gr.target, gr.bin_area / gr.mov_area, self._p(e["map"]),
                    self._p(e["scratch"]), ctypes.c_void_p(out.data_ptr() + 8), s)
        self.sync()
        h = out.cpu().numpy()
        return float(h[0]), float(h[1])

    def tension_unit(self, pos):
        """(#pins / L1 norm over the cells of the plain density gradient at pos, overflow at pos): the unit the
        density weight is given in (Objective.tension_unit, src/calculator.py:20-24) and the overflow of the same
        density pass (density.forward(pos)[1])."""
        out = self.eval(pos, self.tmp[0], weight=1.0, precond=-1.0, with_wl=False)
        return float(self.p.total_pins) / float(out[4]), float(out[3]) * self.overflow_scale()

    def hpwl(self, pos):
        """HPWL of the optimised nets at pos (wirelength.forward(pos, wa_coeff)[2])."""
        with torch.cuda.stream(self.stream):
            self.kp[0] = 10 * self.p.base_gamma
        return float(self.eval(pos, self.tmp[0], weight=0.0, with_wl=True)[2])

    def _passes_left(self, Sh):
        """Passes until the earliest stop the state makes certain, or None: once the run has settled (overflow under
        the target after min_iter), the control stops ("converged") when settled exceeds settle_iter, at the earliest
        after settle_iter + 1 - settled more passes; and at inner_iter passes in all. The host then runs exactly those
        passes instead of a whole batch of check_every; passes after a stop change nothing, so the result is the
        same, with fewer of them computed."""
        o = self.p.opts
        left = [int(o.inner_iter) - int(Sh[SK["loop_it"]])]
        if Sh[SK["settled"]] > 0:
            left.append(int(o.settle_iter) + 1 - int(Sh[SK["settled"]]))
        return max(min(left), 1)

    def _handover_bound(self, Sh):
        """A lower bound on the passes before a run on clusters stops for the hand-over (its smoothing down to
        handover_gamma), or None when that stop is not bounded: with the accuracy rule a pass changes the smoothing by a
        factor within [1/m, m], m = max(mu, 1/mu) <= 1.05 (mu within [1.05 x 0.95, 1.05]), so the smoothing needs at
        least log(gam / handover_gamma) / log(1.05) more passes to reach it."""
        if self.handover_gamma <= 0 or Sh[SK["lam"]] <= 0 or self.p.opts.wa_rule != "accuracy":
            return None
        g = float(Sh[SK["gam"]])
        if g <= self.handover_gamma:
            return 1
        return max(int(math.log(g / self.handover_gamma) / math.log(1.0501)), 1)

    # ------------------------------------------------------------------ one level
    def run(self, pos0, log=None, resume=None):
        """Place from pos0 ([num_nodes, 2], host or device) to the stop. -> dict (reason, iters, start_iters, hpwl,
        overflow, evals, seconds, pos = final positions on the device, iter, lam, gam).
        resume: dict(lam, gam, iter, hpwl, first_iter) to go on where a run on the clusters stopped
        (ParamScheduler.resume, src/param_scheduler.py:53-60; _place_level from first_iter, src/run_placement.py:41):
        the density weight lam and smoothing gam carried over, the scheduler's iteration count and last HPWL, the
        loop counted on from first_iter; no wirelength-only start while lam > 0.
        The phases are also separate calls (begin, the start phase's passes, start_end, the density phase's passes,
        end), which a batch of instances in one graph uses (batch.py)."""
        ctx = self.begin(pos0, resume)
        if ctx["start"]:
            while True:
                self._replay(native.PHASE_START)
                self.sync()
                Th = self.T.cpu().numpy()
                if Th[TI["done"]] or Th[TI["stop"]]:
                    break
            out = self.start_end(ctx, log)
            if out is not None:
                return out
        self._density_loop(ctx, log)
        return self.end(ctx)

    def begin(self, pos0, resume=None):
        """The part before the passes: positions clamped into the region, then the level's set-up on the device
        (gp103_begin: the two probe steps of the step length, estimate_initial_learning_rate and
        NesterovOptimizer.__init__, four gradient evaluations, and the state of the first phase: T of the
        wirelength-only start, or S when resumed with the density term on), with no host synchronisation unless
        resumed. -> context dict."""
        t0 = time.time()
        r = resume or {}
        lam0 = float(r.get("lam", 0.0))
        gam = float(r["gam"]) if resume else self.start_gamma
        first = int(r.get("first_iter", 0))
        self.load(pos0)
        args = self.begin_args(gam, lam0, int(r.get("iter", 0)), first, float(r.get("hpwl", 0.0)))
        native.call("gp103_begin", self._ref, ctypes.byref(args), self._p(self.tmp[0]), self._p(self.tmp[1]),
                    self._p(self.scal), self.stream.cuda_stream)
        ctx = self.context(t0, gam, lam0)
        if lam0 > 0:
            self.check_device("the level's set-up")           # (synchronises the stream)
            ctx.update(it0=first, start_iters=0)
        return ctx

    def context(self, t0, gam=None, lam0=0.0):
        """The context of a run that gp103_begin set up: its start time, WA smoothing, the four gradient evaluations of
        the probes, and whether the wirelength-only start comes first (a fresh run by default)."""
        return dict(t0=t0, gam=self.start_gamma if gam is None else gam, evals=4, start=lam0 <= 0)

    def load(self, pos0):
        """v[0] = pos0 ([num_nodes, 2], host or device) clamped into the region, queued on the Placer's stream."""
        with torch.cuda.stream(self.stream):
            v = self.V[0]
            v.copy_(torch.as_tensor(pos0, dtype=torch.float32).to(self.dev, non_blocking=True))
            torch.max(torch.min(v, self.hi), self.lo, out=v)

    def begin_args(self, gam, lam0=0.0, it=0, first=0, hpwl_prev=0.0):
        """The scalars of gp103_begin: a fresh run by default (lam0 0, the scheduler's iteration count 0)."""
        o = self.p.opts
        return native.BeginArgs(lr=float(o.lr), gamma=float(gam), lam=float(lam0), start_tol=float(o.start_tol),
                                inner_iter=float(o.inner_iter), iter=float(it), loop_it=float(first),
                                hpwl_prev=float(hpwl_prev))

    def start_end(self, ctx, log=None):
        """After the wirelength-only start's passes: the density phase's state. -> None, or the result dict when the
        start phase itself stopped the run."""
        Th = self.T.cpu().numpy()
        out = self.start_over(ctx, Th)
        if out is not None:
            return out
        self.hand_over(ctx)
        if log:
            log("wirelength-only start over after %d iterations (hpwl %.4E): density weight %.4E"
                % (ctx["start_iters"], Th[TI["hpwl"]], float(self.S[SK["lam"]].cpu())))
        return None

    def start_over(self, ctx, Th):
        """The host's part of the end of the start phase, from its final state Th (T on the host): -> the result dict
        when the start phase stopped the run, else None, with ctx set for the density phase."""
        ctx["evals"] += int(Th[TI["evals"]])
        start_iters = int(Th[TI["loop_it"]])
        if Th[TI["stop"]] == STOP_DEVICE_ERROR:
            self.check_device("wirelength-only start")
        if Th[TI["stop"]]:
            reason = REASON[int(Th[TI["stop"]])]
            cur = int(self.cur.cpu())
            return dict(reason=reason, iters=start_iters, start_iters=start_iters, hpwl=float(Th[TI["hpwl"]]),
                        overflow=float("nan"), evals=ctx["evals"], seconds=time.time() - ctx["t0"], pos=self.V[cur],
                        iter=int(Th[TI["iter"]]), lam=0.0, gam=ctx["gam"], density_iters=0)
        ctx.update(it0=start_iters, start_iters=start_iters)
        return None

    def hand_over(self, ctx):
        """Queue the hand-over to the density phase (gp103_start_to_density, no host synchronisation): the first
        density weight, density_weight x the tension unit at the current positions (src/run_placement.py:60-64,
        Objective.tension_unit), and the density phase's state S, kp and best, all set on the device from T."""
        native.call("gp103_start_to_density", self._ref, float(self.p.opts.density_weight), float(self.p.total_pins),
                    float(ctx["gam"]), self._p(self.tmp[0]), self._p(self.scal), self.stream.cuda_stream)

    def _density_loop(self, ctx, log=None):
        o = self.p.opts
        logged = ctx["it0"] // o.log_freq
        # Batches of passes, each followed by an asynchronous copy of the state into pinned memory. While no stop can
        # come within two batches, the next batch is queued before the host waits for the state of the last one, so
        # the GPU does not idle through the poll; near a predictable stop the host runs exactly the passes left. Near a
        # possible hand-over (its bound below two batches) no batch is queued ahead: a queued batch after the stop
        # would be check_every passes that change nothing; below one batch the host runs just the bound's passes and
        # polls again, so that no pass runs past the hand-over.
        inflight, launched = [], [0]

        def launch(k, sort=True):
            if k is None:
                self._replay(native.PHASE_DENSITY)
            else:
                self._passes(native.PHASE_DENSITY, k, sort=sort)  # up to the predicted stop, eagerly
            buf, ev = self._s_host[launched[0] % 2]               # (at most two batches are in flight)
            launched[0] += 1
            with torch.cuda.stream(self.stream):
                buf.copy_(self.S, non_blocking=True)
                ev.record(self.stream)
            inflight.append((buf, ev))

        left, hand = None, None
        launch(None)
        while True:
            if ((left is None or left >= 2 * self.check_every) and (hand is None or hand >= 2 * self.check_every)
                    and len(inflight) < 2):
                launch(None)
            sbuf, ev = inflight.pop(0)
            ev.synchronize()
            Sh = sbuf.numpy().copy()
            left = self._passes_left(Sh)
            hand = self._handover_bound(Sh)
            if not Sh[SK["stop"]] and not inflight:
                if left < self.check_every:
                    launch(left)                                   # exactly the passes to a certain stop
                elif hand is not None and hand < self.check_every:
                    launch(hand, sort=False)                       # no further than the hand-over's lower bound
                else:
                    launch(None)
            it = int(Sh[SK["loop_it"]])
            if log and it // o.log_freq > logged:
                logged = it // o.log_freq
                log("iter: %d | hpwl: %.4E overflow: %.4f density_weight: %.4E wa_coeff: %.4E"
                    % (it, Sh[SK["res_hpwl"]], Sh[SK["res_ovf"]], Sh[SK["lam"]], Sh[SK["gam"]]))
            if Sh[SK["stop"]]:
                break

    def end(self, ctx):
        """After the density phase's passes: the pending best placement, the result dict."""
        native.call("gp103_finish", self._ref, self.stream.cuda_stream)     # (after any batch still queued)
        self.sync()
        Sh = self.S.cpu().numpy()
        if Sh[SK["stop"]] == STOP_DEVICE_ERROR:
            self.check_device("density phase")
        cur = int(self.cur.cpu())
        pos = self.best if Sh[SK["has_best"]] else self.V[cur]
        return dict(reason=REASON[int(Sh[SK["stop"]])], iters=int(Sh[SK["loop_it"]]), start_iters=ctx["start_iters"],
                    hpwl=float(Sh[SK["res_hpwl"]]), overflow=float(Sh[SK["res_ovf"]]),
                    evals=ctx["evals"] + int(Sh[SK["evals"]]), seconds=time.time() - ctx["t0"], pos=pos,
                    density_iters=int(Sh[SK["loop_it"]]) - ctx["it0"], lam=float(Sh[SK["lam"]]),
                    gam=float(Sh[SK["gam"]]), iter=int(Sh[SK["iter"]]))
