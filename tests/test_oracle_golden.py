"""The oracle against the golden fixtures made from AutoPlace's own PyTorch operators (tests/golden/make_golden.py).

These pin the oracle: every later parity test of the CUDA path compares with the oracle."""
import math

import numpy as np
import pytest

from autoplace_gb300 import problem, synth
from oracle import gp_oracle as O


def test_csr_bit_exact(gold):
    g = gold("golden_wa.npz")
    cs = problem.build_csr(g["pin_cell"], g["pin_off"], g["pin_net"], int(g["num_nets"]), int(g["num_mov"]), 100)
    for k in ("net_start", "cell_start", "cell_pin", "cell32"):
        assert np.array_equal(getattr(cs, k), g[k]), k
    assert np.array_equal(cs.off, g["off_opt"])
    assert cs.num_nets == len(g["net_start"]) - 1


@pytest.mark.parametrize("k", [0, 1])
def test_wa_matches_reference(gold, k):
    g = gold("golden_wa.npz")
    n = int(g["num_mov"])
    wa, grad, hpwl, out, _ = O.wa_forward(g["pos"], g["cell32"], g["off_opt"], g["net_start"], n, float(g["gamma%d" % k]))
    ref = g["grad%d" % k]
    assert abs(wa - float(g["wa%d" % k])) <= 1e-5 * abs(wa)
    assert abs(hpwl - float(g["hpwl%d" % k])) <= 1e-6 * hpwl
    assert np.linalg.norm(grad - ref) <= 1e-5 * np.linalg.norm(ref)


def test_exact_hpwl(gold):
    g = gold("golden_wa.npz")
    ns = np.searchsorted(g["pin_net"], np.arange(int(g["num_nets"]) + 1))
    h = O.hpwl_all(g["pos"], g["pin_cell"], g["pin_off"], ns, int(g["num_mov"]))
    assert abs(h - float(g["hpwl_all"])) <= 1e-6 * h


def _grid(g, nb=32, judge=False):
    n = int(g["num_mov"])
    if judge:
        return problem.make_grid(float(g["width"]), float(g["height"]), nb, nb, g["judge_fraction"], float(g["target"]),
                                 g["node_size"][:n], n)
    return problem.make_grid(float(g["width"]), float(g["height"]), nb, nb, g["fixed_fraction"], float(g["target"]),
                             g["node_size"], n)


def test_smoothing_bit_exact(gold):
    g = gold("golden_density.npz")
    gr = _grid(g)
    for a, b in ((gr.size, "smooth_size"), (gr.ratio, "smooth_ratio"), (gr.pos_lo, "pos_lo"), (gr.pos_hi, "pos_hi"),
                 (gr.fixed_map, "fixed_map")):
        assert np.array_equal(a, g[b]), b
    j = _grid(g, 16, judge=True)
    assert np.array_equal(j.size, g["judge_size"]) and np.array_equal(j.ratio, g["judge_ratio"])


def test_density_map_and_overflow(gold):
    g = gold("golden_density.npz")
    gr = _grid(g)
    n = int(g["num_mov"])
    m = O.density_map(g["pos"], gr.size, gr.ratio, n, gr.bx, gr.by, 32, 32)
    rho, over, s = O.density_post(m, gr.fixed_map, gr.target, 32, 32)
    # the reference's CPU path sums node pieces in float32: equal up to that rounding
    assert np.abs(rho - g["mirrored"]).max() <= 1e-5 * max(1.0, np.abs(g["mirrored"]).max())
    assert abs(s * gr.bin_area / gr.mov_area - float(g["overflow_force"])) <= 1e-5
    # a fixed-point map is the same integers whatever the order of the nodes (cells and fillers each shuffled)
    rng = np.random.default_rng(0)
    perm = np.concatenate([rng.permutation(n), n + rng.permutation(len(g["pos"]) - n)])
    m2 = O.density_map(g["pos"][perm], gr.size[perm], gr.ratio[perm], n, gr.bx, gr.by, 32, 32)
    assert np.array_equal(m, m2)


def test_overflow_grid(gold):
    g = gold("golden_density.npz")
    j = _grid(g, 16, judge=True)
    n = int(g["num_mov"])
    mj = O.density_map(g["judge_pos"], j.size, j.ratio, n, j.bx, j.by, 16, 16)
    _, _, s = O.density_post(mj, j.fixed_map, j.target, 16, 16, mirrored=False)
    assert abs(s * j.bin_area / j.mov_area - float(g["judge_overflow"])) <= 1e-5
    real = O.density_map(g["judge_pos"], g["node_size"][:n].astype(np.float32), np.ones(n, np.float32), n, j.bx, j.by,
                         16, 16)
    _, _, s = O.density_post(real, j.fixed_map, j.target, 16, 16, mirrored=False)
    assert abs(s * j.bin_area / j.mov_area - float(g["judge_exact_overflow"])) <= 1e-5


def test_field_fft_and_dct(gold):
    g = gold("golden_density.npz")
    gr = _grid(g)
    op = O.spectral_operator(32, 32, gr.bin_np)
    assert np.abs(op - g["to_field"]).max() <= 1e-6 * np.abs(op).max()
    f64 = O.field_fft(g["mirrored"], 32, 32, gr.bin_np)
    scale = np.abs(f64).max()
    assert np.abs(f64 - g["field"]).max() <= 2e-6 * scale          # the reference computes it in float32
    ex, ey = O.field_dct(g["mirrored"][:32, :32], gr.bin_np)
    assert np.abs(ex - f64[0, :32, :32]).max() <= 1e-12 * scale
    assert np.abs(ey - f64[1, :32, :32]).max() <= 1e-12 * scale


def test_density_gradient(gold):
    g = gold("golden_density.npz")
    gr = _grid(g)
    ex, ey = O.field_dct(g["mirrored"][:32, :32], gr.bin_np)
    grad = O.density_grad(g["pos"], gr.size, gr.ratio, ex, ey, g["wl_grad"], g["pins"], g["area"], 0.37, 0.37, gr.bx,
                          gr.by, 32, 32)
    assert np.linalg.norm(grad - g["grad"]) <= 1e-5 * np.linalg.norm(g["grad"])
    plain = O.density_grad(g["pos"], gr.size, gr.ratio, ex, ey, None, g["pins"], g["area"], 1.0, -1.0, gr.bx, gr.by,
                           32, 32)
    assert np.linalg.norm(plain - g["plain_grad"]) <= 1e-5 * np.linalg.norm(g["plain_grad"])
    # the mirrored layout (row stride 2 nby) reads the same numbers
    f64 = O.field_fft(g["mirrored"], 32, 32, gr.bin_np)
    g2 = O.density_grad(g["pos"], gr.size, gr.ratio, f64[0], f64[1], g["wl_grad"], g["pins"], g["area"], 0.37, 0.37,
                        gr.bx, gr.by, 32, 32)
    assert np.abs(g2 - grad).max() <= 1e-9 * np.abs(grad).max()


def _control_state(g, accuracy):
    S = np.zeros(len(O.FIELDS))
    base = float(g["base_gamma"])
    S[O.K["lam"]], S[O.K["gam"]], S[O.K["alpha"]], S[O.K["a"]] = float(g["lam0"]), 10 * base, 1.0, 1.0
    S[O.K["iter"]], S[O.K["hpwl_prev"]], S[O.K["mu"]] = float(g["iter0"]), float(g["hpwl0"]), 1.0
    S[O.K["best_hpwl"]] = S[O.K["best_ovf"]] = math.inf
    c = np.array([base, float(g["pitch"]) * math.sqrt(float(g["num_nodes"])), float(g["total_pins"]),
                  float(g["total_area"]), float(g["pitch"]), float(g["min_iter"]), float(g["stop_overflow"]),
                  float(g["settle_iter"]), float(g["stall_iter"]), 1e9, float(g["refine"]), float(accuracy), 0.0])
    return S, c


@pytest.mark.parametrize("accuracy", [True, False])
def test_control_matches_param_scheduler(gold, accuracy):
    g = gold("golden_control.npz")
    rows = g["rows"][g["accuracy"] == accuracy]
    S, c = _control_state(g, accuracy)
    kp = np.zeros(5, np.float32)
    K = O.K
    for r in rows:
        k, hpwl, ovf, moved, wa, lam, gam, mu, motion, ww, settled, bh, bo, isb, imp, it, code = r
        O.control(S, kp, c, moved, 1.0, hpwl, ovf, wa)
        for name, want in (("lam", lam), ("gam", gam), ("mu", mu), ("motion", motion), ("ww", ww), ("best_hpwl", bh),
                           ("best_ovf", bo)):
            assert S[K[name]] == pytest.approx(want, rel=1e-12, abs=0), (k, name)
        assert (S[K["settled"]], S[K["is_best"]], S[K["improved"]], S[K["iter"]]) == (settled, isb, imp, it), k
        assert S[K["stop"]] == code, k
        assert kp[0] == np.float32(gam) and kp[1] == np.float32(lam)
    assert S[K["stop"]] != 0          # the sequences end on a stop rule


def test_control_divergence_and_freeze():
    S = np.zeros(len(O.FIELDS))
    S[O.K["gam"]] = S[O.K["a"]] = S[O.K["alpha"]] = 1.0
    S[O.K["best_hpwl"]] = S[O.K["best_ovf"]] = math.inf
    c = np.array([1.0, 10.0, 100.0, 100.0, 1.0, 0, 0.07, 3, 50, 1e9, 1.0, 1.0, 0.0])
    kp = np.zeros(5, np.float32)
    O.control(S, kp, c, 1.0, 2.0, 100.0, 0.5, 90.0)
    assert S[O.K["accept"]] == 1 and S[O.K["stop"]] == 0 and S[O.K["alpha"]] == 0.5
    before = S.copy()
    O.control(S, kp, c, 1.0, float("nan"), 100.0, 0.5, 90.0)       # a step that is not finite is not taken
    assert S[O.K["stop"]] == 3 and S[O.K["accept"]] == 0 and S[O.K["alpha"]] == before[O.K["alpha"]]
    frozen = S.copy()
    O.control(S, kp, c, 1.0, 2.0, 100.0, 0.5, 90.0)                 # stopped: nothing changes any more
    assert np.array_equal(S, frozen)


def test_cpu_placement_matches_reference(gold):
    """The oracle's CPU iteration runs the whole level like the reference (same stop, iterations, HPWL)."""
    g = gold("golden_place.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=0, seed=int(g["seed"]))
    prob = problem.Problem(nl, problem.options(target_density=1.0, num_bin=int(g["num_bin"]), inner_iter=3000))
    assert prob.force_bin == int(g["force_bin"])
    r = O.CpuLevel(prob).run(g["pos0"])
    assert r["reason"] == str(g["reason"]) and r["start_iters"] == int(g["start_iters"])
    assert abs(r["iters"] - int(g["iters"])) <= 5
    h = O.hpwl_all(r["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert abs(h - float(g["hpwl"])) <= 0.005 * float(g["hpwl"])


def test_cluster_matches_reference(gold):
    """cluster_cells (src/cluster.py:38-85): the pair edges and, with the reference's own head draws, every cluster
    and its area."""
    g = gold("golden_cluster.npz")
    i, j, w = O.cluster_edges(g["pin_cell"], g["pin_net"], int(g["n"]))
    assert np.array_equal(i, g["edge_i"]) and np.array_equal(j, g["edge_j"]) and np.array_equal(w, g["edge_w"])
    cid, area = O.cluster_cells(g["pin_cell"], g["pin_net"], g["area"], int(g["ratio"]), lambda r, num: g["draw%d" % r])
    assert np.array_equal(cid, g["cid"]) and np.array_equal(area, g["carea"])
    assert len(area) < int(g["n"]) and int(area.sum()) == int(g["area"].sum())


def _coarse_case(g):
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=int(g["macros"]),
                            cover=float(g["cover"]), fixed_pin_share=float(g["fixed_pin_share"]), seed=int(g["seed"]))
    opts = problem.options(target_density=float(g["target_density"]), num_bin=int(g["num_bin"]),
                           force_num_bin=int(g["force_num_bin"]), cluster_ratio=float(g["cluster_ratio"]),
                           seed=int(g["cluster_seed"]))
    return nl, problem.Problem(nl, opts)


def test_coarse_problem_and_expand_match_reference(gold):
    """coarse_problem (src/cluster.py:88-130: clusters, their sizes and pins) and expand (:133-144), with the
    reference's own generator draws."""
    torch = pytest.importorskip("torch")
    g = gold("golden_coarse.npz")
    nl, prob = _coarse_case(g)
    n = nl.num_mov
    size = np.asarray(prob.node_size[:n], np.float32)
    area = np.round((size[:, 0] * size[:, 1]).astype(np.float64) * 1024).astype(np.int64)
    gen = torch.Generator().manual_seed(int(g["cluster_seed"]))
    cid, carea = O.cluster_cells(nl.pin_cell, nl.pin_net, area, float(g["cluster_ratio"]),
                                 lambda r, num: torch.rand(num, generator=gen).numpy())
    assert np.array_equal(cid, g["cid"]) and len(carea) == int(g["num"])
    num = len(carea)
    single = np.bincount(cid, minlength=num) == 1
    c, off, net = O.coarse_pins(nl.pin_cell, nl.pin_off, nl.pin_net, n, cid, num, single)
    assert np.array_equal(c, g["pin_cell"]) and np.array_equal(net, g["pin_net"])
    assert np.array_equal(off.view(np.uint32), g["pin_off"].view(np.uint32))
    gen = torch.Generator().manual_seed(int(g["cluster_seed"]))
    csize = np.asarray(g["size"], np.float32)
    pos = O.expand(g["cpos"], cid, csize, size, torch.rand(n, 2, generator=gen).numpy(), num)
    assert np.array_equal(pos.view(np.uint32), g["pos"].view(np.uint32))


def test_two_levels_match_reference(gold):
    """The oracle's two-level run (clusters until the hand-over smoothing, expand, the density weight in tension
    units, the cells resumed) and the reference's own (golden_place2.npz): the same clusters and cluster grid, the
    same stop, the clusters' iterations within 3, the total within 5, HPWL within 0.5 %."""
    pytest.importorskip("torch")
    g = gold("golden_place2.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=0, seed=int(g["seed"]))
    prob = problem.Problem(nl, problem.options(target_density=1.0, num_bin=int(g["num_bin"]), force_num_bin=0,
                                               cluster_ratio=float(g["cluster_ratio"]), inner_iter=3000,
                                               seed=int(g["cluster_seed"])))
    r = O.two_level(prob, g["pos0"])
    assert r["clusters"] == int(g["clusters"]) and r["coarse_num_bin"] == int(g["coarse_num_bin"])
    assert r["coarse_reason"] == "handover" and abs(r["coarse_iters"] - int(g["coarse_iters"])) <= 3
    assert r["reason"] == str(g["reason"]) and abs(r["iters"] - int(g["iters"])) <= 5
    h = O.hpwl_all(r["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert abs(h - float(g["hpwl"])) <= 0.005 * float(g["hpwl"])
