"""Two-level placement, step 1: the cells merged into clusters by rounds of star matching, on the device.

Mirrors cluster_cells (src/cluster.py:38-85) call for call: the pair edges of the small nets, then up to
`max_rounds` rounds, each with half of the clusters drawn as heads from a seeded CPU generator (torch.rand of
torch.Generator().manual_seed(seed), as the reference draws them), until the clusters are few enough or a round
merges nothing. The edge building and every round run in libgp103 (gp103_cluster_edges / _round / _relabel); the
host draws the heads and reads two counts per round. Integer weights and areas and fixed tie rules make the result
the reference's, bit for bit.
"""
import ctypes

import numpy as np
import torch

from . import native


def pair_bound(pin_net, max_degree=8):
    """Number of ordered pin pairs of the nets of 2 .. max_degree pins: a bound on the pair entries."""
    deg = np.bincount(np.asarray(pin_net, np.int64))
    d = deg[(deg >= 2) & (deg <= max_degree)].astype(np.int64)
    return int((d * (d - 1)).sum())


def cluster_cells(pin_cell, pin_net, area, ratio, seed, max_degree=8, per_head=3, max_rounds=12, device="cuda",
                  draws=None, stream=None):
    """pin_cell / pin_net [P] sorted by net (cell index len(area) = a fixed pin); area [n] int64. -> (cluster of
    every cell [n] int64, area of every cluster [K] int64), as numpy arrays. draws(round, num) -> float32 [num] can
    stand in for the seeded generator (tests)."""
    area = np.ascontiguousarray(area, np.int64)
    n = len(area)
    if n == 0:
        return np.zeros(0, np.int64), area
    dev = torch.device(device)
    stream = stream or torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    big = 20 * int(area.sum()) // n
    small = area < big
    cap = 3 * int(ratio) * int(area[small].sum()) // (2 * int(small.sum()))
    pin_net = np.asarray(pin_net, np.int64)
    num_nets = int(pin_net.max()) + 1 if len(pin_net) else 0
    E = max(pair_bound(pin_net, max_degree), 1)
    with torch.cuda.stream(stream):
        pc = torch.as_tensor(np.asarray(pin_cell, np.int32)).to(dev)
        pn = torch.as_tensor(pin_net.astype(np.int32)).to(dev)
        scratch = torch.empty(int(native.lib().gp103_cluster_scratch(n, num_nets, E)), dtype=torch.uint8, device=dev)
        rows = [torch.zeros(n + 1, dtype=torch.int32, device=dev) for _ in range(2)]
        col = [torch.zeros(E, dtype=torch.int32, device=dev) for _ in range(2)]
        wgt = [torch.zeros(E, dtype=torch.int32, device=dev) for _ in range(2)]
        areas = [torch.as_tensor(area).to(dev), torch.zeros(n, dtype=torch.int64, device=dev)]
        counts = torch.zeros(2, dtype=torch.int32, device=dev)
        new_index = torch.zeros(n, dtype=torch.int32, device=dev)
        cid = torch.arange(n, dtype=torch.int32, device=dev)
    native.call("gp103_cluster_edges", p(pc), p(pn), len(pin_net), num_nets, n, max_degree, E, p(scratch),
                scratch.numel(), p(rows[0]), p(col[0]), p(wgt[0]), p(counts), s)
    stream.synchronize()
    if int(counts[1]) > E:
        raise RuntimeError("pair bound too small: %d > %d" % (int(counts[1]), E))
    gen = torch.Generator().manual_seed(int(seed))
    num, a = n, 0
    for r in range(max_rounds):
        if num * ratio <= n:
            break
        d = draws(r, num) if draws is not None else torch.rand(num, generator=gen)
        head = torch.as_tensor(np.asarray(d) < np.float32(0.5)).to(torch.uint8)
        with torch.cuda.stream(stream):
            head = head.to(dev)
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
    stream.synchronize()
    return cid.cpu().numpy().astype(np.int64), areas[a][:num].cpu().numpy()
