"""The fused iteration and the whole level on the GPU against the oracle and the reference's golden run."""
import math

import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _problem(cells=12000, nb=128, judge=64, seed=9, macros=5):
    nl = synth.make_netlist(cells, int(cells * 1.05), window=150, macros=macros, cover=0.12, fixed_pin_share=0.02,
                            seed=seed)
    return problem.Problem(nl, problem.options(target_density=0.9, num_bin=judge, force_num_bin=nb))


def _positions(prob, seed=0):
    rng = np.random.default_rng(seed)
    nl, gr = prob.nl, prob.force
    pos = rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]
    pos[: prob.num_mov // 4] = pos[: prob.num_mov // 4] * 0.05 + [nl.width * 0.3, nl.height * 0.6]
    return np.clip(pos, gr.pos_lo, gr.pos_hi).astype(np.float32)


@pytest.mark.parametrize("field,tol", [("bf16x6", 1e-5), ("f16x3", 1e-5), ("fp32", 1e-5), ("bf16x3", 1e-4),
                                       ("tf32x3", 1e-5)])
def test_fused_gradient_matches_oracle(field, tol):
    from autoplace_gb300.engine import Placer
    prob = _problem()
    pl = Placer(prob, field=field)
    pos = torch.tensor(_positions(prob), device="cuda")
    out = torch.zeros_like(pos)
    gam, lam = 37.5, 3.1e-4
    pl.kp[0] = gam
    r = pl.eval(pos, out, weight=lam, precond=lam, with_wl=True)
    og, owa, ohpwl, oovf = O.CpuLevel(prob).grad(pos.cpu().numpy(), lam, gam)
    assert relerr(out.cpu().numpy(), og) <= tol
    assert abs(r[1] - owa) <= 1e-6 * abs(owa) and abs(r[2] - ohpwl) <= 1e-6 * ohpwl
    assert abs(r[3] * pl.overflow_scale() - oovf) <= 1e-6
    # the wirelength-only gradient and the plain density gradient of tension_unit
    r0 = pl.eval(pos, out, weight=0.0, with_wl=True)
    og0 = O.CpuLevel(prob).grad(pos.cpu().numpy(), 0.0, gam)[0]
    assert relerr(out.cpu().numpy(), og0) <= 1e-5
    r1 = pl.eval(pos, out, weight=1.0, precond=-1.0, with_wl=False)
    tu = O.CpuLevel(prob).tension_unit(pos.cpu().numpy())
    assert abs(prob.pins.sum() / r1[4] - tu) <= 1e-5 * tu


def test_fused_pass_is_repeatable():
    from autoplace_gb300.engine import Placer
    prob = _problem(cells=6000, nb=128, judge=64, seed=3)
    res = []
    for _ in range(2):
        pl = Placer(prob, field="bf16x6", check_every=8)
        r = pl.run(synth.init_positions(prob.nl, prob.num_nodes, seed=1))
        res.append((r["iters"], r["hpwl"], r["overflow"], r["pos"].cpu().numpy()))
    assert res[0][:3] == res[1][:3]
    assert np.array_equal(res[0][3], res[1][3])


def test_split_pass_matches_single_stream():
    """The WA kernels on a second stream beside the density map and the field (gp103_pass_split), joined before the
    gather or before the field (GP103_PASS_JOIN_FIELD): the same run, bit for bit, graphs or not."""
    from autoplace_gb300.engine import Placer
    prob = _problem(cells=6000, nb=128, judge=64, seed=3)
    pos0 = synth.init_positions(prob.nl, prob.num_nodes, seed=1)
    res = []
    for split, graphs in ((False, True), (True, True), (True, False), ("field", True), ("field", False)):
        r = Placer(prob, field="f16x3", check_every=8, split=split, use_graphs=graphs).run(pos0)
        res.append((r["iters"], r["hpwl"], r["overflow"], r["pos"].cpu().numpy()))
    for r in res[1:]:
        assert r[:3] == res[0][:3]
        assert np.array_equal(r[3], res[0][3])


def test_side_stream_never_the_pass_stream():
    """torch hands out streams round robin from a small pool: however many were drawn before, a split Placer's side
    stream is not its own stream (gp103_pass_split refuses side == stream)."""
    from autoplace_gb300.engine import side_stream
    s = torch.cuda.Stream()
    for _ in range(100):
        assert side_stream(s).cuda_stream != s.cuda_stream


def test_level_matches_reference_run(gold):
    """The reference's own CPU run (golden_place.npz) and this GPU run of the same level: same stop, HPWL within
    0.5 %, iteration counts within 5 %."""
    from autoplace_gb300.engine import Placer
    g = gold("golden_place.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=0, seed=int(g["seed"]))
    prob = problem.Problem(nl, problem.options(target_density=1.0, num_bin=int(g["num_bin"]), inner_iter=3000))
    r = Placer(prob, field="fp32").run(g["pos0"])
    pos = r["pos"].cpu().numpy()
    h = O.hpwl_all(pos, prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert r["reason"] == str(g["reason"])
    assert r["start_iters"] == int(g["start_iters"])
    assert abs(r["iters"] - int(g["iters"])) <= 0.05 * int(g["iters"])
    assert abs(h - float(g["hpwl"])) <= 0.005 * float(g["hpwl"])


@pytest.mark.parametrize("field", ["bf16x6", "f16x3", "bf16x3", "tf32x3"])
def test_level_matches_oracle_with_tensor_core_field(field):
    """10,000 cells on a 128 x 128 force grid: GPU run (tensor-core field) vs the oracle's CPU run."""
    from autoplace_gb300.engine import Placer
    nl, o = synth.preset("c0")
    prob = problem.Problem(nl, problem.options(**o))
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    r = Placer(prob, field=field).run(pos0)
    ref = O.CpuLevel(prob).run(pos0)
    assert r["reason"] == ref["reason"] == "converged"
    h = O.hpwl_all(r["pos"].cpu().numpy(), prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    hr = O.hpwl_all(ref["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert abs(h - hr) <= 0.005 * hr
    assert r["overflow"] < 0.07


def test_divergence_keeps_last_finite_point():
    """A gradient that is not finite (injected on the host between graph replays) makes the next step non-finite:
    the control stops with 'diverged' and the current placement stays the last finite one."""
    from autoplace_gb300 import native
    from autoplace_gb300.engine import Placer, SK
    prob = _problem(cells=4000, nb=128, judge=64, seed=5, macros=2)
    pl = Placer(prob, field="bf16x6", check_every=4, use_graphs=False)
    r = pl.run(synth.init_positions(prob.nl, prob.num_nodes, seed=2))
    assert r["reason"] in ("converged", "stalled")
    # restart the density phase by hand from the stopped state with a poisoned gradient (the finiteness test
    # comes before every stop rule)
    S = pl.S.cpu().numpy()
    S[SK["stop"]] = 0
    S[SK["loop_it"]] = 0
    pl.S.copy_(torch.as_tensor(S))
    cur = int(pl.cur.cpu())
    before = pl.V[cur].clone()
    pl.G[cur][7, 0] = float("nan")
    pl._passes(native.PHASE_DENSITY, 3)
    pl.sync()
    S = pl.S.cpu().numpy()
    assert S[SK["stop"]] == 3 and int(pl.cur.cpu()) == cur
    assert torch.equal(pl.V[cur], before) and bool(torch.isfinite(pl.V[cur]).all())


def _two_level_case(g):
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=0, seed=int(g["seed"]))
    opts = problem.options(target_density=1.0, num_bin=int(g["num_bin"]), force_num_bin=0,
                           cluster_ratio=float(g["cluster_ratio"]), inner_iter=3000, seed=int(g["cluster_seed"]))
    return problem.Problem(nl, opts)


@pytest.mark.parametrize("graphs", [True, False])
def test_two_levels_match_reference_run(gold, graphs):
    """The reference's own two-level run (golden_place2.npz: the clusters placed until the hand-over smoothing, then
    the cells) and this GPU run (global_placement, src/run_placement.py:79-122): the same clusters (integer work,
    exact) and cluster grid, the same stop, the clusters' iterations within 3, the total within 5 %, HPWL within
    0.5 %, overflow within 0.005."""
    from autoplace_gb300.flow import global_placement
    g = gold("golden_place2.npz")
    prob = _two_level_case(g)
    st = global_placement(prob, g["pos0"], field="fp32", use_graphs=graphs)
    assert st["clusters"] == int(g["clusters"]) and st["coarse_num_bin"] == int(g["coarse_num_bin"])
    assert abs(st["coarse_iters"] - int(g["coarse_iters"])) <= 3
    assert st["stop_reason"] == str(g["reason"])
    assert abs(st["iters"] - int(g["iters"])) <= 0.05 * int(g["iters"])
    hpwl, ovf = st["placer"].evaluate(st["pos"])
    assert abs(hpwl - float(g["hpwl"])) <= 0.005 * float(g["hpwl"])
    assert abs(ovf - float(g["overflow"])) <= 0.005


def test_two_levels_single_level_when_ratio_is_one(gold):
    """cluster_ratio 1: global_placement is one level of the cells, as Placer.run."""
    from autoplace_gb300.engine import Placer
    from autoplace_gb300.flow import global_placement
    g = gold("golden_place2.npz")
    prob = _two_level_case(g)
    prob.opts.cluster_ratio = 1.0
    st = global_placement(prob, g["pos0"], field="fp32")
    r = Placer(prob, field="fp32").run(g["pos0"])
    assert "clusters" not in st and st["iters"] == r["iters"] and st["stop_reason"] == r["reason"]
    assert np.array_equal(st["pos"].cpu().numpy(), r["pos"].cpu().numpy())


def test_c0_two_levels_match_oracle_with_tensor_core_field():
    """The 10,000-cell netlist as its configuration states it: cluster_ratio 5 (the reference's default, two levels),
    the cells' 128 x 128 force grid in f16x3 on the tensor cores (the clusters' smaller grid in fp32), against the
    oracle's two-level CPU run (float64, the field as cosine transforms): the same clusters and cluster grid, the
    same stop, HPWL within 0.5 %, and the control's overflow under the stop target."""
    from autoplace_gb300.flow import global_placement
    nl, o = synth.preset("c0")
    prob = problem.Problem(nl, problem.options(**o))
    assert prob.opts.cluster_ratio == 5.0
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    st = global_placement(prob, pos0, field="f16x3")
    assert st["placer"].mode == native.FIELD_F16X3
    ref = O.two_level(prob, pos0)
    assert st["clusters"] == ref["clusters"] and st["coarse_num_bin"] == ref["coarse_num_bin"]
    assert st["stop_reason"] == ref["reason"] == "converged"
    h = O.hpwl_all(st["pos"].cpu().numpy(), prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    hr = O.hpwl_all(ref["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert abs(h - hr) <= 0.005 * hr, (h, hr)
    assert st["overflow"] < prob.opts.stop_overflow
    assert abs(st["iters"] - ref["iters"]) <= 0.1 * ref["iters"], (st["iters"], ref["iters"])
