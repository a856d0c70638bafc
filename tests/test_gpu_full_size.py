"""The kernels at the size of the 1.2M-cell workload (1,200,000 cells, 1,250,000 nets, 5,209,352 pins, 40 macros,
173,979 fillers; force grid 1024 x 1024, overflow grid 512 x 512), checked through what does not depend on size:

  - integer work bit for bit: the fixed-point density map and its post-processing against the oracle's C
    restatement (at the start, where every cell sits in one small cloud, and on a spread placement with a clump),
    the problem build and the WA net order on the device against the host build;
  - float work against the oracle in float64, with the tolerances of the small cases (the float32 restatement of the
    same arithmetic stays within 1.6e-6 of float64 here): WA gradient and per-net values, the field gather, the
    exact HPWL and overflow;
  - a whole placement: two runs, and a run of the device-built problem, end at the same positions bit for bit (fixed
    reduction orders), stop by the overflow rule, and the exact judges agree with the control's own numbers.
"""
import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from oracle import gp_oracle as O
from tests.test_gpu_ops import _native_map, cu, gp_cuda, relerr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def c2():
    nl, o = synth.preset("c2", seed=0)
    prob = problem.Problem(nl, problem.options(**o))
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    return nl, prob, pos0


def _spread(nl, prob, seed=11):
    """Nodes uniform over the region, a third of the cells clumped into a spot of 1 % of the region's side."""
    gr = prob.force
    rng = np.random.default_rng(seed)
    pos = (rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]).astype(np.float32)
    k = nl.num_mov // 3
    pos[:k] = pos[:k] * np.float32(0.01) + np.array([nl.width * 0.4, nl.height * 0.55], np.float32)
    return np.clip(pos, gr.pos_lo, gr.pos_hi).astype(np.float32)


# ------------------------------------------------------------------------------------------------ integer work
@pytest.mark.parametrize("start", [True, False])
def test_full_size_density_map_bit_exact(c2, start):
    nl, prob, pos0 = c2
    gr = prob.force
    pos = np.clip(pos0, gr.pos_lo, gr.pos_hi).astype(np.float32) if start else _spread(nl, prob)
    m, rho, over = _native_map(pos, gr.size, gr.ratio, prob.num_mov, gr)
    om = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    assert np.array_equal(m, om)
    orho, oover, _ = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    assert np.array_equal(rho.view(np.uint32), orho.view(np.uint32))
    assert np.array_equal(over.view(np.uint32), oover.view(np.uint32))


def test_full_size_device_build_and_net_order_match_host(c2):
    from tests.test_gpu_setup import _check_device_problem, device_order
    from autoplace_gb300.engine import net_order
    nl, prob, _ = c2
    _check_device_problem(nl, prob.opts)
    cs = prob.csr
    perm, new_start, slot, *bounds = net_order(cs.net_start, cs.cell32, cs.cell_pin)
    ns_d, cell_d, off_d, slot_d, split_d = device_order(cs, nl.num_mov)
    assert np.array_equal(ns_d, new_start)
    assert np.array_equal(cell_d, cs.cell32[perm])
    assert np.array_equal(off_d.view(np.uint32), cs.off[perm].view(np.uint32))
    assert np.array_equal(slot_d, slot)
    assert split_d == list(bounds)


# ------------------------------------------------------------------------------------------------ float work
@pytest.mark.parametrize("gamma_scale", [10.0, 1.0])
def test_full_size_wa_matches_oracle(c2, gamma_scale):
    nl, prob, _ = c2
    cs = prob.csr
    pos = _spread(nl, prob)
    gamma = gamma_scale * prob.base_gamma
    grad, out = gp_cuda().wa(cu(pos), cu(cs.cell32), cu(cs.off), cu(cs.net_start), cu(cs.cell_start),
                             cu(cs.cell_pin), nl.num_mov, cu(np.array([gamma], np.float32)))
    wa, ograd, hpwl, oout, _ = O.wa_forward(pos, cs.cell32, cs.off, cs.net_start, nl.num_mov, gamma)
    grad, out = grad.cpu().numpy(), out.cpu().numpy()
    assert relerr(grad, ograd) <= 1e-5
    assert np.abs(out[:, 1] - oout[:, 1]).max() <= 1e-6 * np.abs(oout[:, 1]).max()
    assert np.abs(out[:, 0] - oout[:, 0]).max() <= 1e-5 * np.abs(oout[:, 0]).max()
    tot = out.astype(np.float64).sum(0)
    assert abs(tot[0] - wa) <= 1e-5 * abs(wa) and abs(tot[1] - hpwl) <= 1e-6 * hpwl


def test_full_size_density_grad_matches_oracle(c2):
    nl, prob, _ = c2
    gr = prob.force
    pos = _spread(nl, prob)
    om = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    orho, _, _ = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    field = O.field_fft(orho, gr.nbx, gr.nby, gr.bin_np)
    wl = np.random.default_rng(2).standard_normal((prob.num_mov, 2)).astype(np.float32)
    weight, precond = 0.37, 0.37
    grad = gp_cuda().density_grad(cu(pos), cu(gr.size), cu(gr.ratio), cu(field.astype(np.float32)), cu(wl),
                                  cu(prob.pins), cu(prob.area), cu(np.array([weight], np.float32)),
                                  cu(np.array([precond], np.float32)), gr.bx, gr.by, gr.nbx, gr.nby)
    og = O.density_grad(pos, gr.size, gr.ratio, field[0], field[1], wl, prob.pins, prob.area, weight, precond,
                        gr.bx, gr.by, gr.nbx, gr.nby)
    assert relerr(grad.cpu().numpy(), og) <= 1e-5


def _oracle_judges(nl, prob, pos):
    gr = prob.real_judge
    C = prob.num_mov
    hpwl = O.hpwl_all(pos, prob.all_cell, prob.all_off, prob.all_net_start, C)
    size = np.ascontiguousarray(nl.size, dtype=np.float32)
    om = O.density_map(pos[:C], size, np.ones(C, np.float32), C, gr.bx, gr.by, gr.nbx, gr.nby)
    _, _, total = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby, mirrored=False)
    return hpwl, total * gr.bin_area / gr.mov_area


# ------------------------------------------------------------------------------------------------ a placement
def test_full_size_placement_is_deterministic_and_judged_exactly(c2):
    from autoplace_gb300.engine import Placer
    nl, prob, pos0 = c2
    pl = Placer(prob)
    r1 = pl.run(pos0)
    p1 = r1["pos"].cpu().numpy()
    r2 = pl.run(pos0)
    assert r1["reason"] == r2["reason"] == "converged" and r1["iters"] == r2["iters"]
    assert np.array_equal(p1.view(np.uint32), r2["pos"].cpu().numpy().view(np.uint32))
    assert r1["overflow"] <= prob.opts.stop_overflow
    # the exact judges (float64 on the device) against the oracle at the final placement
    hpwl, ovf = pl.evaluate(r1["pos"])
    ohpwl, oovf = _oracle_judges(nl, prob, p1)
    assert abs(hpwl - ohpwl) <= 1e-11 * ohpwl and abs(ovf - oovf) <= 1e-11 * max(oovf, 1e-30)
    # every net of this netlist is optimised (degree <= 100): the control's HPWL is the exact one in float32 sums
    assert abs(r1["hpwl"] - hpwl) <= 1e-5 * hpwl
    del pl
    # the problem built on the device from the netlist's arrays places to the same positions
    dp = problem.Problem(nl, prob.opts, arrays=False).on_device()
    r3 = Placer(dp).run(pos0)
    assert r3["iters"] == r1["iters"]
    assert np.array_equal(r3["pos"].cpu().numpy().view(np.uint32), p1.view(np.uint32))


# ------------------------------------------------------------------------------------------------ field precision
def _states(nl, prob, pos0):
    """Density states of a real placement of this netlist: the start (every cell in a cloud of 0.1 % of the region's
    side, its hottest bins far above the target), a state mid-run (the run cut at 150 iterations, overflow still
    high), and the final placement."""
    import copy
    from autoplace_gb300.engine import Placer
    gr = prob.force
    out = {"start": np.clip(pos0, gr.pos_lo, gr.pos_hi).astype(np.float32)}
    mid = copy.copy(prob)
    mid.opts = problem.options(**dict(vars(prob.opts), inner_iter=150))
    r = Placer(mid).run(pos0)
    assert r["reason"] == "max_iter"
    out["mid"] = r["pos"].cpu().numpy()
    out["final"] = Placer(prob).run(pos0)["pos"].cpu().numpy()
    return out


@pytest.fixture(scope="module")
def c2_states(c2):
    nl, prob, pos0 = c2
    return _states(nl, prob, pos0)


@pytest.mark.parametrize("state", ["start", "mid", "final"])
@pytest.mark.parametrize("mode,tol", [(native.FIELD_F16X3, 1e-6), (native.FIELD_BF16X6, 1e-6),
                                      (native.FIELD_TF32X3, 1e-6)])
def test_full_size_field_error_on_real_states(c2, c2_states, state, mode, tol):
    """The tensor-core field of the 1024 x 1024 force grid against float64 (the cosine-transform statement of the
    reference's mirrored FFT) on the densities of a real run: max |E - E64| / max |E64| <= 1e-6. The density plane
    is the run's own (the float32 total density of the fixed-point map), with the Placer's shift (the grid's mean
    density, taken off before the transforms: the same field, rounding relative to the density's variation)."""
    import ctypes
    from autoplace_gb300.engine import mean_density
    from tests.test_gpu_ops import _field_plan
    nl, prob, _ = c2
    gr = prob.force
    pos = c2_states[state]
    _, rho, _ = _native_map(pos, gr.size, gr.ratio, prob.num_mov, gr)
    a = np.ascontiguousarray(rho[:gr.nbx, :gr.nby])
    pl, keep = _field_plan(gr.nbx, mode, bx=gr.bx, by=gr.by)
    pl.field_shift = mean_density(prob)            # as the Placer sets it: the grid's mean density
    ex, ey = torch.zeros((gr.nbx, gr.nby), device=DEV), torch.zeros((gr.nbx, gr.nby), device=DEV)
    d = cu(a)
    native.call("gp103_field", ctypes.byref(pl), d.data_ptr(), ex.data_ptr(), ey.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    fx, fy = O.field_dct(a, gr.bin_np)
    scale = max(np.abs(fx).max(), np.abs(fy).max())
    err = max(np.abs(ex.cpu().numpy() - fx).max(), np.abs(ey.cpu().numpy() - fy).max()) / scale
    print("field error %s mode %d: %.3e (peak density %.4g)" % (state, mode, err, a.max()))
    assert err <= tol, err
