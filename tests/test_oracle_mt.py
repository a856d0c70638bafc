"""The oracle's multi-threaded operators (oracle/level_ref.c, used by the CPU level on the host cores) against its
single-threaded restatement: the same integer map, the same gather, and WA in float32 within float32 rounding of
the numpy float32 statement (exponentials by the C library instead of numpy's)."""
import numpy as np

from autoplace_gb300 import problem, synth
from oracle import gp_oracle as O


def _case(seed=4):
    nl = synth.make_netlist(6000, 6300, window=100, macros=3, cover=0.1, fixed_pin_share=0.02, seed=seed)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=64, force_num_bin=128))
    rng = np.random.default_rng(seed)
    pos = rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]
    pos[:1500] = pos[:1500] * 0.05 + [nl.width * 0.3, nl.height * 0.6]
    return prob, np.clip(pos, prob.force.pos_lo, prob.force.pos_hi).astype(np.float32)


def test_mt_operators_match_single_threaded():
    prob, pos = _case()
    O.set_threads(4)
    gr, cs = prob.force, prob.csr
    m1 = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    m4 = O.density_map_mt(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    assert np.array_equal(m1, m4)
    rho, _, _ = O.density_post(m1, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    fx, fy = O.field_fft(rho, gr.nbx, gr.nby, gr.bin_np)
    wl = np.random.default_rng(1).standard_normal((prob.num_mov, 2)).astype(np.float32)
    g1 = O.density_grad(pos, gr.size, gr.ratio, fx, fy, wl, prob.pins, prob.area, 0.3, 0.3, gr.bx, gr.by, gr.nbx,
                        gr.nby)
    g4 = O.density_grad_mt(pos, gr.size, gr.ratio, fx, fy, wl, prob.pins, prob.area, 0.3, 0.3, gr.bx, gr.by,
                           gr.nbx, gr.nby)
    assert np.array_equal(g1, g4)
    for gamma in (40.0, 3.0):
        # float32 WA loses about |x| / gamma x 1e-7 in (x - mean) / gamma: both float32 statements are judged against
        # float64, the threaded one no worse than twice the numpy one's error
        wa, grad, hpwl, out, pg = O.wa_forward(pos, cs.cell32, cs.off, cs.net_start, prob.num_mov, gamma, np.float32)
        wa8, grad8, hpwl8, out8, pg8 = O.wa_forward(pos, cs.cell32, cs.off, cs.net_start, prob.num_mov, gamma)
        wa4, grad4, hpwl4, out4, pg4 = O.wa_forward_mt(pos, cs.cell32, cs.off, cs.net_start, cs.cell_start,
                                                       cs.cell_pin, prob.num_mov, gamma)
        for mine, np32, ref in ((pg4, pg, pg8), (grad4, grad, grad8)):
            e_np = np.abs(np32 - ref).max()
            assert np.abs(mine - ref).max() <= 2 * e_np + 1e-6 * np.abs(ref).max()
        assert np.array_equal(out4[:, 1], out[:, 1])               # HPWL: max - min, no rounding choice
        assert abs(wa4 - wa8) <= 2 * abs(wa - wa8) + 1e-6 * abs(wa8) and abs(hpwl4 - hpwl8) <= 1e-6 * hpwl8


def test_mt_fft_field_matches_numpy():
    prob, pos = _case(5)
    gr = prob.force
    m = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    rho, _, _ = O.density_post(m, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    a = O.field_fft(rho, gr.nbx, gr.nby, gr.bin_np, np.float32)
    b = O.field_fft(rho, gr.nbx, gr.nby, gr.bin_np, np.float32, workers=4)
    c = O.field_fft(rho, gr.nbx, gr.nby, gr.bin_np)
    assert np.abs(b - c).max() <= 1e-5 * np.abs(c).max()
    assert np.abs(a - c).max() <= 1e-5 * np.abs(c).max()


def test_mt_level_runs_like_the_numpy_level():
    """A whole small level on 4 threads (float32 WA, FFT field) ends like the single-threaded float32 level: same
    stop reason, iterations within 5 %, HPWL within 0.5 %."""
    nl = synth.make_netlist(3000, 3150, window=80, macros=2, cover=0.1, fixed_pin_share=0.02, seed=6)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=32, force_num_bin=64))
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=6)
    a = O.CpuLevel(prob, dtype=np.float32, field="fft").run(pos0)
    b = O.CpuLevel(prob, dtype=np.float32, field="fft", threads=4).run(pos0)
    assert a["reason"] == b["reason"] == "converged"
    assert abs(a["iters"] - b["iters"]) <= 0.05 * a["iters"]
    ha = O.hpwl_all(a["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    hb = O.hpwl_all(b["pos"], prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    assert abs(ha - hb) <= 0.005 * ha
