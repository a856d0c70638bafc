"""ORACLE — test infrastructure only.

CPU statement of the learned start's network (autoplace_gb300/learn.py, csrc/learn.cu) with torch autograd as the
checker of its hand-written forward and backward kernels: the same graph operators (mean of a net's movable pins'
clusters, then mean of a cluster's nets), the same layers, bf16-rounded weights and fp32 arithmetic, the mean squared
error against targets. Also the cluster features (anchor propagation from the fixed pins) in numpy.

The reference has no learned part: this restates the network's definition, not reference code. Only tests/ import
this module.
"""
import math

import numpy as np
import torch

LAYERS, WIDTH = 3, 64


def graph_ops(net_start, pin_cell, cell_start, cell_pin, K):
    """(P2N as (net, cluster, weight) triples, N2C as (cluster, net, weight) triples) of the pins: numpy arrays."""
    net_start = np.asarray(net_start, np.int64)
    pin_cell = np.asarray(pin_cell, np.int64)
    N = len(net_start) - 1
    pin_net = np.repeat(np.arange(N), np.diff(net_start))
    mov = pin_cell < K
    cnt = np.bincount(pin_net[mov], minlength=N).astype(np.float64)
    inv = np.where(cnt > 0, 1.0 / np.maximum(cnt, 1), 0.0)
    p2n = (pin_net[mov], pin_cell[mov], inv[pin_net[mov]])
    cs = np.asarray(cell_start, np.int64)
    deg = np.diff(cs).astype(np.float64)
    cells = np.repeat(np.arange(K), np.diff(cs))
    pins = np.asarray(cell_pin, np.int64)[:cs[-1]]          # (the fixed pins come after the last cell's)
    n2c = (cells, pin_net[pins], 1.0 / np.maximum(deg[cells], 1))
    return p2n, n2c, N


def _agg(h, p2n, n2c, N, K):
    r, c, w = p2n
    m = torch.zeros((N, h.shape[1]), dtype=h.dtype).index_add_(0, torch.as_tensor(r),
                                                               h[torch.as_tensor(c)] * torch.as_tensor(w, dtype=h.dtype)[:, None])
    r, c, w = n2c
    return torch.zeros((K, h.shape[1]), dtype=h.dtype).index_add_(0, torch.as_tensor(r),
                                                                  m[torch.as_tensor(c)] * torch.as_tensor(w, dtype=h.dtype)[:, None])


def bf16(a):
    return torch.as_tensor(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float32)


def forward_backward(params, x, target, net_start, pin_cell, cell_start, cell_pin, K):
    """-> (y [K, 2], loss, grads {name: array}) of the network with bf16-rounded weights (fp32 biases), fp32 math;
    the gradients are those of the rounded weights (the optimiser applies them to the fp32 master copy)."""
    p2n, n2c, N = graph_ops(net_start, pin_cell, cell_start, cell_pin, K)
    leaves = {}
    for k, v in params.items():
        t = bf16(v) if k[0] in "WSN" else torch.as_tensor(np.asarray(v, np.float32))
        leaves[k] = t.clone().requires_grad_(True)
    x = torch.as_tensor(np.asarray(x, np.float32))
    h = torch.relu(x @ leaves["W0"] + leaves["b0"])
    for l in range(LAYERS):
        a = _agg(h, p2n, n2c, N, K)
        h = torch.relu(h @ leaves["S%d" % l] + a @ leaves["N%d" % l] + leaves["b%d" % (l + 1)])
    y = torch.sigmoid(h @ leaves["Wo"] + leaves["bo"])
    t = torch.as_tensor(np.asarray(target, np.float32))
    loss = ((y - t) ** 2).sum(1).mean()
    loss.backward()
    return y.detach().numpy(), float(loss.detach()), {k: v.grad.numpy() for k, v in leaves.items()}


def features(net_start, pin_cell, pin_off, cell_start, cell_pin, K, area, pin_count, width, height, max_hop=12,
             sweeps=64):
    """The 10 features of each cluster (gp103_learn_features) in float64: log(area / mean), log(1 + nets) / 4,
    log(1 + member pins) / 4, the anchor (x, y as fractions of the region: at hop 0 the mean of the fixed pins of the
    cluster's nets, then the mean over the anchored clusters of each net, averaged over the cluster's nets), hop /
    max_hop, anchored, the anchor's distance from the centre, the harmonic x and y (from the anchors, `sweeps` Jacobi
    sweeps: a net's mean over all its pins, a fixed pin where it is, then a cluster's mean over its nets)."""
    net_start = np.asarray(net_start, np.int64)
    pin_cell = np.asarray(pin_cell, np.int64)
    off = np.asarray(pin_off, np.float64)
    N = len(net_start) - 1
    pin_net = np.repeat(np.arange(N), np.diff(net_start))
    fixed = pin_cell >= K
    fc = np.bincount(pin_net[fixed], minlength=N).astype(np.float64)
    fx = np.bincount(pin_net[fixed], weights=off[fixed, 0], minlength=N)
    fy = np.bincount(pin_net[fixed], weights=off[fixed, 1], minlength=N)
    r = np.zeros((N, 3))
    has = fc > 0
    r[has, 0] = fx[has] / fc[has] / width
    r[has, 1] = fy[has] / fc[has] / height
    r[has, 2] = 1.0
    p2n, n2c, _ = graph_ops(net_start, pin_cell, cell_start, cell_pin, K)

    def n2c_mean(v):
        rr, cc, ww = n2c
        out = np.zeros((K, 3))
        np.add.at(out, rr, v[cc] * ww[:, None])
        return out

    def p2n_mean(v):
        rr, cc, ww = p2n
        out = np.zeros((N, 3))
        np.add.at(out, rr, v[cc] * ww[:, None])
        return out

    anc = np.zeros((K, 3))
    hops = np.full(K, -1.0)
    for hop in range(max_hop + 1):
        z = n2c_mean(r if hop == 0 else p2n_mean(anc))
        new = (hops < 0) & (z[:, 2] > 0)
        anc[new, 0] = z[new, 0] / z[new, 2]
        anc[new, 1] = z[new, 1] / z[new, 2]
        anc[new, 2] = 1.0
        hops[new] = hop
    nets = np.diff(np.asarray(cell_start, np.int64)).astype(np.float64)
    area = np.asarray(area, np.float64)
    ax = np.where(hops >= 0, anc[:, 0], 0.5)
    ay = np.where(hops >= 0, anc[:, 1], 0.5)
    h = np.stack([ax, ay], 1)
    deg = np.diff(net_start).astype(np.float64)
    fixed_xy = np.stack([off[:, 0] / width, off[:, 1] / height], 1)
    for _ in range(sweeps):
        pin_xy = np.where(fixed[:, None], fixed_xy, h[np.minimum(pin_cell, K - 1)])
        r = np.zeros((N, 3))
        np.add.at(r[:, :2], pin_net, pin_xy)
        r[:, :2] /= np.maximum(deg, 1)[:, None]
        r[:, 2] = deg > 0
        z = n2c_mean(r)
        upd = z[:, 2] > 0
        h[upd] = z[upd, :2] / z[upd, 2:3]
    return np.stack([np.log(area / area.mean()), np.log1p(nets) / 4, np.log1p(np.asarray(pin_count, np.float64)) / 4,
                     ax, ay, np.where(hops >= 0, hops / max_hop, 1.0), (hops >= 0).astype(np.float64),
                     np.sqrt((ax - 0.5) ** 2 + (ay - 0.5) ** 2), h[:, 0], h[:, 1]], 1)
