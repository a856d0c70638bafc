"""Clustering on the device (gp103_cluster_*) against the reference's own output (golden_cluster.npz) and against
the oracle's restatement on larger netlists: integer work, so bit for bit."""
import ctypes

import numpy as np
import pytest

from autoplace_gb300 import cluster, native, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _edges(pin_cell, pin_net, n):
    E = max(cluster.pair_bound(pin_net), 1)
    num_nets = int(np.max(pin_net)) + 1
    pc = torch.as_tensor(np.asarray(pin_cell, np.int32)).cuda()
    pn = torch.as_tensor(np.asarray(pin_net, np.int32)).cuda()
    scratch = torch.empty(int(native.lib().gp103_cluster_scratch(n, num_nets, E)), dtype=torch.uint8, device="cuda")
    rows = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    col = torch.zeros(E, dtype=torch.int32, device="cuda")
    w = torch.zeros(E, dtype=torch.int32, device="cuda")
    counts = torch.zeros(2, dtype=torch.int32, device="cuda")
    native.call("gp103_cluster_edges", pc.data_ptr(), pn.data_ptr(), len(pin_net), num_nets, n, 8, E,
                scratch.data_ptr(), scratch.numel(), rows.data_ptr(), col.data_ptr(), w.data_ptr(), counts.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    m = int(counts[0])
    r = rows.cpu().numpy()
    i = np.repeat(np.arange(n), np.diff(r))
    return i, col.cpu().numpy()[:m], w.cpu().numpy()[:m], int(counts[1]), E


@pytest.mark.parametrize("seed", [0, 1, 12345, 2**40 + 7])
def test_seeded_uniform_matches_torch_cpu(seed):
    """gp103_seeded_uniform: torch.rand's CPU stream of a seeded generator (MT19937, 24-bit floats), the same bits, at
    counts on both sides of the 624-word state and at millions of values; consecutive calls continue one stream."""
    for count in (1, 623, 624, 625, 3 * 624 + 5, 2_000_003):
        dev = cluster.seeded_uniform(seed, count).cpu().numpy()
        ref = torch.rand(count, generator=torch.Generator().manual_seed(seed)).numpy()
        assert np.array_equal(dev, ref), (seed, count)
    g = torch.Generator().manual_seed(seed)
    two = np.concatenate([torch.rand(1000, generator=g).numpy(), torch.rand(500, 2, generator=g).numpy().ravel()])
    assert np.array_equal(cluster.seeded_uniform(seed, 2000).cpu().numpy(), two)


def test_pair_edges_match_reference(gold_cluster):
    g = gold_cluster
    i, j, w, found, E = _edges(g["pin_cell"], g["pin_net"], int(g["n"]))
    assert found <= E
    assert np.array_equal(i, g["edge_i"]) and np.array_equal(j, g["edge_j"]) and np.array_equal(w, g["edge_w"])


def test_clusters_match_reference(gold_cluster):
    g = gold_cluster
    cid, area = cluster.cluster_cells(g["pin_cell"], g["pin_net"], g["area"], int(g["ratio"]), int(g["seed"]),
                                      draws=lambda r, num: g["draw%d" % r])
    assert np.array_equal(cid, g["cid"]) and np.array_equal(area, g["carea"])
    # the seeded generator of the product path draws the same heads as the reference did
    cid2, area2 = cluster.cluster_cells(g["pin_cell"], g["pin_net"], g["area"], int(g["ratio"]), int(g["seed"]))
    assert np.array_equal(cid2, g["cid"]) and np.array_equal(area2, g["carea"])


@pytest.mark.parametrize("cells,seed,ratio", [(30000, 2, 5), (12000, 9, 2)])
def test_clusters_match_oracle(cells, seed, ratio):
    nl = synth.make_netlist(cells, int(cells * 1.05), window=300, macros=2, cover=0.1, fixed_pin_share=0.05, seed=seed)
    area = np.round(nl.size.prod(1) * 1024).astype(np.int64)
    gen = torch.Generator().manual_seed(seed)
    cache = {}

    def draws(r, num):
        if r not in cache:
            cache[r] = torch.rand(num, generator=gen).numpy()
        return cache[r]

    ocid, oarea = O.cluster_cells(nl.pin_cell, nl.pin_net, area, ratio, draws)
    cid, carea = cluster.cluster_cells(nl.pin_cell, nl.pin_net, area, ratio, seed, draws=draws)
    assert np.array_equal(cid, ocid) and np.array_equal(carea, oarea)
    assert len(carea) < cells and int(carea.sum()) == int(area.sum())


def test_coarse_problem_and_expand_match_reference(gold):
    """The cluster problem built on the device (clusters, sizes, pins, grid, smoothed nodes, totals) and expand."""
    from autoplace_gb300 import problem
    g = gold("golden_coarse.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=int(g["macros"]),
                            cover=float(g["cover"]), fixed_pin_share=float(g["fixed_pin_share"]), seed=int(g["seed"]))
    opts = problem.options(target_density=float(g["target_density"]), num_bin=int(g["num_bin"]),
                           force_num_bin=int(g["force_num_bin"]), cluster_ratio=float(g["cluster_ratio"]),
                           seed=int(g["cluster_seed"]))
    prob = problem.Problem(nl, opts)
    coarse = cluster.coarse_problem(prob, build="host")
    cp = coarse.problem
    assert np.array_equal(coarse.cid, g["cid"]) and coarse.num == int(g["num"])
    assert np.array_equal(coarse.size.view(np.uint32), np.asarray(g["size"], np.float32).view(np.uint32))
    assert np.array_equal(cp.nl.pin_cell, g["pin_cell"]) and np.array_equal(cp.nl.pin_net, g["pin_net"])
    assert np.array_equal(np.asarray(cp.nl.pin_off, np.float32).view(np.uint32), g["pin_off"].view(np.uint32))
    assert cp.force_bin == int(g["nbx"]) and cp.num_nodes == int(g["num_nodes"])
    assert np.array_equal(cp.force.size.view(np.uint32), g["smooth_size"].view(np.uint32))
    assert np.array_equal(cp.force.ratio.view(np.uint32), g["smooth_ratio"].view(np.uint32))
    assert np.array_equal(cp.pins.view(np.uint32), g["pins"].view(np.uint32))
    assert np.array_equal(cp.force.fixed_map.view(np.uint32), g["fixed_map"].view(np.uint32))
    assert cp.total_pins == float(g["total_pins"]) and abs(cp.total_area - float(g["total_area"])) <= 1e-9 * cp.total_area
    pos = cluster.expand(g["cpos"], coarse, prob, int(g["cluster_seed"])).cpu().numpy()
    assert np.array_equal(pos.view(np.uint32), g["pos"].view(np.uint32))


def test_coarse_problem_device_build_matches_host(gold):
    """The clusters' problem built on the device from the selected pins (no download) and the host build: the same
    arrays, bit for bit."""
    from autoplace_gb300 import problem
    g = gold("golden_coarse.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=int(g["macros"]),
                            cover=float(g["cover"]), fixed_pin_share=float(g["fixed_pin_share"]), seed=int(g["seed"]))
    opts = problem.options(target_density=float(g["target_density"]), num_bin=int(g["num_bin"]),
                           force_num_bin=int(g["force_num_bin"]), cluster_ratio=float(g["cluster_ratio"]),
                           seed=int(g["cluster_seed"]))
    prob = problem.Problem(nl, opts)
    h = cluster.coarse_problem(prob, build="host").problem
    d = cluster.coarse_problem(prob, build="device").problem
    same = lambda a, b: np.array_equal(np.ascontiguousarray(a.cpu().numpy() if hasattr(a, "cpu") else a).view(np.uint8),
                                       np.ascontiguousarray(b).view(np.uint8))
    assert d.csr.num_nets == h.csr.num_nets and d.total_pins == h.total_pins
    for k in ("net_start", "cell32", "off", "cell_start", "cell_pin"):
        assert same(getattr(d.csr, k), getattr(h.csr, k)), k
    for k in ("all_cell", "all_off", "all_net_start", "pins", "area"):
        assert same(getattr(d, k), getattr(h, k)), k
    for k in ("size", "ratio", "pos_lo", "pos_hi"):
        assert same(getattr(d.force, k), getattr(h.force, k)), k
    assert np.array_equal(d.constants(), h.constants())
