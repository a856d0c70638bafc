"""The learned start: a message-passing network over the cluster graph proposes where the clusters start, in place of
the reference's start (the clusters at the seeded start positions, src/run_placement.py:98, then the wirelength-only
start, src/run_placement.py:48-65 with src/param_scheduler.py:42-48). The reference has no learned part.

Network (3 message-passing layers, hidden width 64, bf16 weights with an fp32 master copy, fp32 accumulation):
    h0      = relu(x W0 + b0)                              x: 10 features per cluster (gp103_learn_features)
    a_l     = N2C(P2N(h_l))                                mean over each net's clusters, then over a cluster's nets
    h_{l+1} = relu(h_l S_l + a_l N_l + b_l),  l = 0, 1, 2
    y       = sigmoid(h3 Wo + bo)                          (x, y) as fractions of the region
Every step is a libgp103 kernel (csrc/learn.cu): the gathers over the cluster netlist's two CSRs (and their
transposes for the backward pass), the dense layers, the loss and the optimiser; training is deterministic.

Training data: placements the method itself makes (the plain two-level flow, tensor-core field) of seeded synthetic
netlists of 5,000-50,000 cells (config-0 generator, 5-30 macros); the target of a cluster is the mean final position
of its cells. Training and inference run on the GPU through the same kernels.

Use: Proposal(load_model()).hook is the `start` of flow.Flow.run: it computes the features of the run's clusters,
runs the network, and starts the clusters' level from the proposed positions with the density term on (no
wirelength-only start), the density weight in tension units as the plain start's first weight times the model's
`lam_scale`. The plain start is the fallback, at two levels: a model is used only when its held-out validation
placements (the plain method's exact HPWL and overflow judging them, both runs at the same stop overflow) kept the
plain start's HPWL within 1 % (the model file's `use`, model_available), and only for designs in the size range it was
trained and validated on (`cells_min` .. `cells_max`, Proposal.applies); and a placement from the proposal that does
not converge is placed again from the plain start (flow.Flow.run(fallback=True)).
"""
import ctypes
import math
import os
import time

import numpy as np
import torch

from . import native, synth

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_FILE = os.path.join(HERE, "start_net.npz")
F_IN, WIDTH, LAYERS, MAX_HOP, SWEEPS = 10, 64, 3, 12, 64
CELLS_MIN, CELLS_MAX = 5000, 50000       # the training generator's design sizes (sample_netlist)
ACT_NONE, ACT_RELU, ACT_SIGMOID = 0, 1, 2

def lib():
    return native.lib()


def _call(name, *args):
    native.check(getattr(lib(), name)(*args), name)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


# ------------------------------------------------------------------------------------------------ the graph
class Graph(object):
    """The cluster netlist as the message passing reads it: the optimised nets of a Problem's csr (device tensors
    or host arrays), pins grouped by net and by cluster, and the weights of the four gathers (csrc/learn.cu)."""

    def __init__(self, csr, num_cells, device="cuda", stream=None):
        dev = torch.device(device)
        self.stream = stream or torch.cuda.current_stream(dev)
        s = self.stream.cuda_stream
        t = lambda a, dt: (a if torch.is_tensor(a) else torch.as_tensor(np.ascontiguousarray(a))).to(
            device=dev, dtype=dt).contiguous()
        with torch.cuda.stream(self.stream):
            self.net_start = t(csr.net_start, torch.int32)
            self.pin_cell = t(csr.cell32, torch.int32)
            self.pin_off = t(csr.off, torch.float32)
            self.cell_start = t(csr.cell_start, torch.int32)
            self.cell_pin = t(csr.cell_pin, torch.int32)
            self.N, self.K, self.P = int(csr.num_nets), int(num_cells), int(self.pin_cell.shape[0])
            P = max(self.P, 1)
            e = lambda dt: torch.empty(P, dtype=dt, device=dev)
            self.net_pin_cell, self.w_p2n, self.w_n2ct = e(torch.int32), e(torch.float32), e(torch.float32)
            self.cell_pin_net, self.w_n2c, self.w_p2nt = e(torch.int32), e(torch.float32), e(torch.float32)
            scratch = torch.empty(int(lib().gp103_learn_graph_scratch(self.N, self.P)), dtype=torch.uint8, device=dev)
        _call("gp103_learn_graph", _p(self.net_start), _p(self.pin_cell), _p(self.cell_start), _p(self.cell_pin),
              self.N, self.K, self.P, _p(scratch), scratch.numel(), _p(self.net_pin_cell), _p(self.w_p2n),
              _p(self.w_n2ct), _p(self.cell_pin_net), _p(self.w_n2c), _p(self.w_p2nt), s)
        self._keep = scratch

    def aggregate(self, h, out_net, out, accumulate=False):
        """out = N2C(P2N(h)) (width of h), through out_net [N, width]."""
        w, s = h.shape[1], self.stream.cuda_stream
        _call("gp103_seg_gather", _p(self.net_start), self.N, _p(self.net_pin_cell), _p(self.w_p2n), _p(h), w, 0,
              _p(out_net), s)
        _call("gp103_seg_gather", _p(self.cell_start), self.K, _p(self.cell_pin_net), _p(self.w_n2c), _p(out_net), w,
              int(accumulate), _p(out), s)

    def aggregate_t(self, d, out_net, out, accumulate=True):
        """out (+)= P2N^T(N2C^T(d)): the transpose of aggregate (the backward pass)."""
        w, s = d.shape[1], self.stream.cuda_stream
        _call("gp103_seg_gather", _p(self.net_start), self.N, _p(self.net_pin_cell), _p(self.w_n2ct), _p(d), w, 0,
              _p(out_net), s)
        _call("gp103_seg_gather", _p(self.cell_start), self.K, _p(self.cell_pin_net), _p(self.w_p2nt), _p(out_net), w,
              int(accumulate), _p(out), s)

    def features(self, area, width, height, pin_count=None, max_hop=MAX_HOP, sweeps=SWEEPS):
        """[K, 10] features (gp103_learn_features): area, nets, member pins, the propagated fixed-pin anchor and its
        hop distance, the harmonic coordinates. area, pin_count: [K] device tensors (float32)."""
        dev = self.net_start.device
        with torch.cuda.stream(self.stream):
            area = area.to(dev, torch.float32).contiguous()
            mean_area = float(area.double().mean()) if self.K else 1.0
            feat = torch.empty((max(self.K, 1), F_IN), dtype=torch.float32, device=dev)
            scratch = torch.empty(int(lib().gp103_learn_features_scratch(self.N, self.K)), dtype=torch.uint8,
                                  device=dev)
            pc = None if pin_count is None else pin_count.to(dev, torch.float32).contiguous()
        _call("gp103_learn_features", _p(self.net_start), _p(self.pin_cell), _p(self.pin_off), _p(self.cell_start),
              self.N, self.K, self.P, _p(self.net_pin_cell), _p(self.w_p2n), _p(self.cell_pin_net), _p(self.w_n2c),
              _p(area), _p(pc), max(mean_area, 1e-30), float(width), float(height), int(max_hop), int(sweeps),
              _p(scratch),
              scratch.numel(), _p(feat), self.stream.cuda_stream)
        return feat[:self.K]


# ------------------------------------------------------------------------------------------------ the network
def _param_shapes():
    shapes = [("W0", (F_IN, WIDTH)), ("b0", (WIDTH,))]
    for l in range(LAYERS):
        shapes += [("S%d" % l, (WIDTH, WIDTH)), ("N%d" % l, (WIDTH, WIDTH)), ("b%d" % (l + 1), (WIDTH,))]
    shapes += [("Wo", (WIDTH, 2)), ("bo", (2,))]
    return shapes


def init_params(seed=0):
    """fp32 parameters {name: array}: He-normal weights, zero biases (the output bias at the region's centre)."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, shape in _param_shapes():
        if len(shape) == 2:
            fan_in = shape[0] * (2 if name.startswith("N") or name.startswith("S") else 1)
            out[name] = (rng.standard_normal(shape) * math.sqrt(2.0 / fan_in)).astype(np.float32)
        else:
            out[name] = np.zeros(shape, np.float32)
    out["Wo"] *= 0.1
    return out


class Net(object):
    """The network's parameters on the device: one flat fp32 buffer (master), its bf16 copy (the weights the kernels
    read) and the Adam moments; named views into each."""

    def __init__(self, params, device="cuda"):
        dev = torch.device(device)
        shapes = _param_shapes()
        sizes = [int(np.prod(s)) for _, s in shapes]
        n = sum(sizes)
        flat = np.concatenate([np.asarray(params[k], np.float32).ravel() for k, _ in shapes])
        self.flat = torch.as_tensor(flat).to(dev)
        self.flat16 = self.flat.to(torch.bfloat16)
        self.grad = torch.zeros(n, dtype=torch.float32, device=dev)
        self.m = torch.zeros(n, dtype=torch.float32, device=dev)
        self.v = torch.zeros(n, dtype=torch.float32, device=dev)
        self.step = 0
        self.views, self.views16, self.gviews = {}, {}, {}
        o = 0
        for (name, shape), k in zip(shapes, sizes):
            self.views[name] = self.flat[o:o + k].view(shape)
            self.views16[name] = self.flat16[o:o + k].view(shape)
            self.gviews[name] = self.grad[o:o + k].view(shape)
            o += k

    def params(self):
        return {k: v.detach().cpu().numpy().copy() for k, v in self.views.items()}

    def adam(self, lr, stream, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step += 1
        _call("gp103_adam", _p(self.flat), _p(self.grad), _p(self.m), _p(self.v), _p(self.flat16),
              int(self.flat.numel()), float(lr), float(beta1), float(beta2), float(eps), self.step,
              float(weight_decay), stream.cuda_stream)


def _dense(x, a, wx, wa, b, out_dim, act, out, stream):
    n, in_x = x.shape
    in_a = 0 if a is None else a.shape[1]
    _call("gp103_dense_fwd", _p(x), n, in_x, _p(a), in_a, _p(wx), _p(wa), _p(b), out_dim, act, _p(out),
          stream.cuda_stream)


class Pass(object):
    """Forward (and backward) passes of the network, one graph at a time, in a workspace for graphs of up to
    max_cells clusters and max_nets nets (the activations of the last forward are kept for its backward)."""

    def __init__(self, net, max_cells, max_nets, stream, device="cuda"):
        self.net, self.stream = net, stream
        dev = torch.device(device)
        K, N = max(int(max_cells), 1), max(int(max_nets), 1)
        self.cap = (K, N)
        with torch.cuda.stream(stream):
            z = lambda *shape: torch.empty(shape, dtype=torch.float32, device=dev)
            self.h = [z(K, WIDTH) for _ in range(LAYERS + 1)]
            self.a = [z(K, WIDTH) for _ in range(LAYERS)]
            self.tmp_net = z(N, WIDTH)
            self.y = z(K, 2)
            self.dh = [z(K, WIDTH) for _ in range(2)]
            self.da = z(K, WIDTH)
            self.dz = z(K, WIDTH)
            self.dy = z(K, 2)
            self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
            self.red = torch.zeros(native.EVAL_SCRATCH_BYTES, dtype=torch.uint8, device=dev)
            self.wscratch = torch.empty(int(lib().gp103_dense_bwd_scratch(WIDTH, WIDTH, WIDTH)), dtype=torch.uint8,
                                        device=dev)
        self.g = None

    @classmethod
    def for_graph(cls, net, g):
        return cls(net, g.K, g.N, g.stream, g.net_start.device)

    def forward(self, g, x):
        """-> y [K, 2]: the proposed positions as fractions of the region (a view into the workspace)."""
        if g.K > self.cap[0] or g.N > self.cap[1]:
            raise ValueError("graph of %d clusters / %d nets beyond the workspace %s" % (g.K, g.N, self.cap))
        self.g = g
        v, s, K, N = self.net.views16, self.stream, g.K, g.N
        b = self.net.views
        _dense(x, None, v["W0"], None, b["b0"], WIDTH, ACT_RELU, self.h[0], s)
        for l in range(LAYERS):
            g.aggregate(self.h[l][:K], self.tmp_net[:N], self.a[l])
            _dense(self.h[l][:K], self.a[l][:K], v["S%d" % l], v["N%d" % l], b["b%d" % (l + 1)], WIDTH, ACT_RELU,
                   self.h[l + 1], s)
        _dense(self.h[LAYERS][:K], None, v["Wo"], None, b["bo"], 2, ACT_SIGMOID, self.y, s)
        return self.y[:K]

    def loss_and_grad(self, g, x, target):
        """Forward, the mean squared error against target [K, 2] (device float64 scalar, self.loss), backward: the
        parameter gradients into net.grad."""
        self.forward(g, x)
        _call("gp103_mse", _p(self.y), _p(target), g.K, 2, _p(self.dy), _p(self.loss), _p(self.red),
              self.stream.cuda_stream)
        self.backward(x)
        return self.loss

    def _dense_bwd(self, x, a, wx, wa, out, dout, dx, da, gwx, gwa, gb, out_dim, act):
        n, in_x = x.shape
        in_a = 0 if a is None else a.shape[1]
        _call("gp103_dense_bwd", _p(x), n, in_x, _p(a), in_a, _p(wx), _p(wa), out_dim, act, _p(out), _p(dout),
              _p(self.dz), _p(dx), _p(da), _p(self.wscratch), self.wscratch.numel(), _p(gwx), _p(gwa), _p(gb),
              self.stream.cuda_stream)

    def backward(self, x):
        v, gv, g = self.net.views16, self.net.gviews, self.g
        K, N = g.K, g.N
        cur = self.dh[LAYERS % 2]
        self._dense_bwd(self.h[LAYERS][:K], None, v["Wo"], None, self.y, self.dy, cur, None, gv["Wo"], None,
                        gv["bo"], 2, ACT_SIGMOID)
        for l in reversed(range(LAYERS)):
            nxt = self.dh[l % 2]
            self._dense_bwd(self.h[l][:K], self.a[l][:K], v["S%d" % l], v["N%d" % l], self.h[l + 1], cur, nxt,
                            self.da, gv["S%d" % l], gv["N%d" % l], gv["b%d" % (l + 1)], WIDTH, ACT_RELU)
            g.aggregate_t(self.da[:K], self.tmp_net[:N], nxt, accumulate=True)
            cur = nxt
        self._dense_bwd(x, None, v["W0"], None, self.h[0], cur, None, None, gv["W0"], None, gv["b0"], WIDTH,
                        ACT_RELU)


# ------------------------------------------------------------------------------------------------ models on disk
def model_available(path=MODEL_FILE):
    """A trained model whose validation kept the plain start's HPWL within 1 % is present."""
    if not os.path.exists(path):
        return False
    return bool(load_model(path).get("use", False))


def load_model(path=MODEL_FILE):
    """-> dict(params={name: fp32 array}, lam_scale, cells_min, cells_max, meta...)."""
    z = np.load(path, allow_pickle=False)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    out = {"params": params, "cells_min": CELLS_MIN, "cells_max": CELLS_MAX}
    for k in z.files:
        if not k.startswith("p_"):
            out[k] = z[k].item() if z[k].shape == () else z[k]
    return out


def save_model(path, params, **meta):
    np.savez(path, **{"p_" + k: np.asarray(v, np.float32) for k, v in params.items()}, **meta)


# ------------------------------------------------------------------------------------------------ the proposal
def cluster_inputs(coarse, prob, device="cuda", stream=None):
    """The features of a run's clusters: (Graph, features [K, 10]) from cluster.coarse_problem's result."""
    cp = coarse.problem
    K = coarse.num
    stream = stream or torch.cuda.current_stream(torch.device(device))
    g = Graph(cp.csr, K, device=device, stream=stream)
    with torch.cuda.stream(stream):
        area = torch.as_tensor(synth.areas(cp.node_size[:K]).astype(np.float32)).to(device)
        # the member cells' pins of each cluster, summed on the device (whole numbers: any order gives the same sums)
        pin_count = torch.zeros(max(K, 1), dtype=torch.float32, device=device)
        pin_count.index_add_(0, coarse.cid_dev.to(device=device, dtype=torch.long), _cell_pins(prob, device))
    x = g.features(area, prob.nl.width, prob.nl.height, pin_count[:K])
    return g, x


def _cell_pins(prob, device):
    """Pins of every movable cell (all nets) as a float32 device tensor, uploaded once per problem."""
    dev = torch.device(device)
    got = prob.__dict__.get("_cell_pins_dev")
    if got is None or got.device != dev:
        got = torch.as_tensor(np.asarray(prob.nl.cell_pins, np.float32)).to(dev)
        prob.__dict__["_cell_pins_dev"] = got
    return got


class Proposal(object):
    """The learned start as a Flow.run `start` hook."""

    def __init__(self, model, device="cuda"):
        self.model = model
        self.cells = (int(model.get("cells_min", CELLS_MIN)), int(model.get("cells_max", CELLS_MAX)))
        self.dev = torch.device(device)
        self.net = Net(model["params"], device=self.dev)
        self.lam_scale = float(model.get("lam_scale", 1.0))
        self.last = None
        self._pass = None           # the forward workspace, kept for the next design of at most its size

    def positions(self, coarse, prob, stream):
        g, x = cluster_inputs(coarse, prob, self.dev, stream)
        ps = self._pass
        if ps is None or ps.stream is not stream or g.K > ps.cap[0] or g.N > ps.cap[1]:
            ps = self._pass = Pass.for_graph(self.net, g)
        y = ps.forward(g, x)
        return y, g

    def applies(self, prob):
        """The model is used for designs of the size range it was trained and validated on (the fallback rule)."""
        return self.cells[0] <= prob.num_mov <= self.cells[1]

    def hook(self, coarse, cplacer, cpos0, prob):
        """-> (cluster + filler positions, resume dict): the clusters at the network's positions (clamped to their
        bounds), the fillers where they were; the clusters' level resumed with the density term on. prob: the
        cells' problem (its netlist's pin counts feed the features)."""
        stream = cplacer.stream
        y, _ = self.positions(coarse, prob, stream)
        K = coarse.num
        with torch.cuda.stream(stream):
            region = torch.tensor([prob.nl.width, prob.nl.height], dtype=torch.float32, device=self.dev)
            pos = cpos0.clone()
            pos[:K] = y * region
            torch.max(torch.min(pos, cplacer.hi), cplacer.lo, out=pos)
        o = cplacer.p.opts
        tu = cplacer.tension_unit(pos)[0]
        lam = self.lam_scale * o.density_weight * tu
        resume = dict(lam=lam, gam=10 * cplacer.p.base_gamma, iter=0, hpwl=cplacer.hpwl(pos), first_iter=0)
        self.last = dict(lam=lam)
        return pos, resume


# ------------------------------------------------------------------------------------------------ training data
def sample_netlist(seed):
    """The seeded training netlist `seed`: the config-0 generator with cells log-uniform in 5,000 .. 50,000, nets
    1.05 x cells, 5 .. 30 macros over 5 .. 20 % of the region, target density 0.75 .. 1.0, two levels (cluster ratio
    5). -> (netlist, options)."""
    from . import problem, synth
    rng = np.random.default_rng(1_000_003 + int(seed))
    cells = int(round(math.exp(rng.uniform(math.log(5000), math.log(50000)))))
    macros = int(rng.integers(5, 31))
    cover = float(rng.uniform(0.05, 0.20))
    target = float(rng.uniform(0.75, 1.0))
    nl = synth.make_netlist(cells, int(round(cells * 1.05)), window=200, macros=macros, cover=cover, seed=int(seed))
    return nl, problem.options(target_density=target, num_bin=0, cluster_ratio=5.0, seed=int(seed))


def _prepare(seed):
    """Host part of a training sample (a worker process): the netlist, its problem, its start positions."""
    from . import problem, synth
    nl, opts = sample_netlist(seed)
    prob = problem.Problem(nl, opts)
    return seed, prob, synth.init_positions(nl, prob.num_nodes, seed=int(seed))


def cluster_targets(coarse, pos, prob):
    """Each cluster's target: the mean position of its cells in `pos` (a placement of the cells), as fractions of the
    region -> float32 [K, 2]."""
    p = np.asarray(pos[:prob.num_mov], np.float64)
    cnt = np.bincount(coarse.cid, minlength=coarse.num).astype(np.float64)
    t = np.stack([np.bincount(coarse.cid, weights=p[:, a], minlength=coarse.num) / cnt for a in range(2)], 1)
    return (t / np.array([prob.nl.width, prob.nl.height])).astype(np.float32)


def make_sample(prob, pos0, field="f16x3", device="cuda"):
    """One placement of the plain method (two levels, the reference's start) -> dict: the cluster graph (host CSR
    arrays), the features and targets of its clusters, and the run's statistics."""
    from .flow import Flow
    flow = Flow(prob, field=field, device=device)
    st = flow.run(pos0)
    coarse = flow.last_coarse
    g, x = cluster_inputs(coarse, prob, device, flow.stream)
    flow.stream.synchronize()
    cs = coarse.problem.csr
    host = lambda a: a.cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    out = dict(net_start=host(cs.net_start).astype(np.int32), pin_cell=host(cs.cell32).astype(np.int32),
               pin_off=host(cs.off).astype(np.float32), cell_start=host(cs.cell_start).astype(np.int32),
               cell_pin=host(cs.cell_pin).astype(np.int32), num_nets=int(cs.num_nets), K=int(coarse.num),
               x=x.cpu().numpy(), target=cluster_targets(coarse, st["pos"].cpu().numpy(), prob),
               iters=int(st["iters"]), coarse_iters=int(st.get("coarse_iters", 0)), seconds=float(st["gp_time_s"]),
               cells=prob.num_mov)
    del flow
    return out


def generate(seeds, field="f16x3", workers=8, log=None):
    """Training samples of the given seeds: netlists and problems built by `workers` host processes (spawned, so
    that they hold no CUDA state), placements on the GPU. -> list of make_sample dicts."""
    import multiprocessing as mp
    out = []
    t0 = time.time()
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        for k, (seed, prob, pos0) in enumerate(pool.imap(_prepare, list(seeds))):
            out.append(make_sample(prob, pos0, field=field))
            if log and (k + 1) % 50 == 0:
                log("samples: %d (%.1fs)" % (k + 1, time.time() - t0))
    return out


# ------------------------------------------------------------------------------------------------ training
class _Sample(object):
    """A training sample on the device: its graph, features and targets."""

    def __init__(self, d, device="cuda", stream=None):
        from types import SimpleNamespace
        csr = SimpleNamespace(net_start=d["net_start"], cell32=d["pin_cell"], off=d["pin_off"],
                              cell_start=d["cell_start"], cell_pin=d["cell_pin"], num_nets=d["num_nets"])
        self.g = Graph(csr, d["K"], device=device, stream=stream)
        with torch.cuda.stream(self.g.stream):
            self.x = torch.as_tensor(d["x"]).to(device)
            self.t = torch.as_tensor(d["target"]).to(device)


def train(samples, epochs=30, lr=2e-3, seed=0, device="cuda", log=None, params=None):
    """Adam on the mean squared error of the proposed positions, one sample (graph) per step, samples in a seeded
    order each epoch, the learning rate decayed by cosine to lr / 20. -> (params, per-epoch mean losses)."""
    stream = torch.cuda.Stream(torch.device(device))
    net = Net(params or init_params(seed), device=device)
    data = [_Sample(d, device, stream) for d in samples]
    work = Pass(net, max(s.g.K for s in data), max(s.g.N for s in data), stream, device)
    rng = np.random.default_rng(seed)
    total = epochs * len(data)
    history = []
    step = 0
    for ep in range(epochs):
        losses = []
        for i in rng.permutation(len(data)):
            rate = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * step / max(total, 1))))
            loss = work.loss_and_grad(data[i].g, data[i].x, data[i].t)
            net.adam(rate, stream)
            losses.append(loss.clone())
            step += 1
        stream.synchronize()
        history.append(float(torch.cat(losses).mean()))
        if log:
            log("epoch %d: loss %.5f" % (ep, history[-1]))
    return net.params(), history


def evaluate_start(seeds, model, lam_scales=(1.0,), field="f16x3", device="cuda", log=None):
    """Plain vs learned starts on held-out netlists: for each seed, the plain two-level placement and the learned one
    at each density-weight scale. -> list of dicts (iterations, seconds, exact HPWL and overflow)."""
    from .flow import Flow
    from . import problem, synth
    rows = []
    for seed in seeds:
        nl, opts = sample_netlist(seed)
        prob = problem.Problem(nl, opts)
        pos0 = synth.init_positions(nl, prob.num_nodes, seed=int(seed))
        flow = Flow(prob, field=field, device=device)
        flow.run(pos0)                                                   # warm-up (graphs)
        row = {"seed": int(seed), "cells": nl.num_mov}
        st = flow.run(pos0)
        h, o = flow.fine.evaluate(st["pos"])
        row["plain"] = dict(iters=st["iters"], seconds=st["gp_time_s"], hpwl=h, overflow=o, reason=st["stop_reason"])
        for ls in lam_scales:
            prop = Proposal(dict(model, lam_scale=ls), device=device)
            flow.run(pos0, start=prop.hook)
            st = flow.run(pos0, start=prop.hook)
            h, o = flow.fine.evaluate(st["pos"])
            row["learned_%g" % ls] = dict(iters=st["iters"], seconds=st["gp_time_s"], hpwl=h, overflow=o,
                                          reason=st["stop_reason"])
        rows.append(row)
        if log:
            log(str(row))
        del flow
    return rows


def main(argv=None):
    """python -m autoplace_gb300.learn train --train 2000 --val 32 --epochs 30 --out start_net.npz"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--train", type=int, default=2000, help="training netlists: seeds 0 .. n-1")
    ap.add_argument("--val", type=int, default=32, help="held-out netlists: seeds 100000 ..")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--workers", type=int, default=max((os.cpu_count() or 2) - 2, 1))
    ap.add_argument("--lam-scales", default="1,3,10,30")
    ap.add_argument("--out", default=MODEL_FILE)
    ap.add_argument("--report", default=None)
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    t0 = time.time()
    samples = generate(range(a.train), workers=a.workers, log=log)
    t_gen = time.time() - t0
    log("generated %d samples in %.1fs" % (len(samples), t_gen))
    t0 = time.time()
    params, hist = train(samples, epochs=a.epochs, lr=a.lr, log=log)
    t_train = time.time() - t0
    scales = [float(x) for x in a.lam_scales.split(",")]
    model = {"params": params}
    rows = evaluate_start(range(100_000, 100_000 + a.val), model, scales, log=log)
    # the density-weight scale: the fastest mean time whose HPWL stays within 1 % of the plain start's on average (the
    # fallback rule: no such scale, or none faster than the plain start -> the model is not used)
    best, best_t, summary = 1.0, None, {}
    for ls in scales:
        k = "learned_%g" % ls
        t = float(np.mean([r[k]["seconds"] / r["plain"]["seconds"] for r in rows]))
        h = float(np.mean([r[k]["hpwl"] / r["plain"]["hpwl"] for r in rows]))
        it = float(np.mean([r[k]["iters"] / r["plain"]["iters"] for r in rows]))
        summary[ls] = (t, h, it)
        log("lam_scale %g: time / plain %.3f, iterations / plain %.3f, hpwl / plain %.4f" % (ls, t, it, h))
        if h <= 1.01 and (best_t is None or t < best_t):
            best, best_t = ls, t
    use = best_t is not None and best_t < 1.0
    t, h, it = summary.get(best, (1.0, 1.0, 1.0))
    save_model(a.out, params, lam_scale=best, use=use, val_time_ratio=t, val_hpwl_ratio=h, val_iter_ratio=it,
               cells_min=min(s["cells"] for s in samples), cells_max=max(s["cells"] for s in samples),
               train_samples=len(samples), epochs=a.epochs, final_loss=hist[-1], gen_seconds=t_gen,
               train_seconds=t_train)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(dict(history=hist, rows=rows, lam_scale=best, gen_seconds=t_gen, train_seconds=t_train,
                           samples=[{k: v for k, v in s.items() if k in ("K", "iters", "coarse_iters", "seconds",
                                                                          "cells")} for s in samples]), f)
    log("saved %s (lam_scale %g)" % (a.out, best))


if __name__ == "__main__":
    main()
