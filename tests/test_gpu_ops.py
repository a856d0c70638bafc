"""Parity of the sm_103a kernels with the oracle, through the C ABI (the gp_cuda drop-in module and libgp103's
own entry points). Integer work (the density map) must be bit-exact; float work within the stated tolerances."""
import ctypes
import math

import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


def cu(a, dt=None):
    t = torch.as_tensor(np.ascontiguousarray(a))
    return (t.to(dt) if dt is not None else t).to(DEV)


def gp_cuda():
    from autoplace_gb300 import gp_cuda as g
    return g


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ------------------------------------------------------------------------------------------------ WA
def _wa_case(nl, gamma, seed=0):
    cs = problem.build_csr(nl.pin_cell, nl.pin_off, nl.pin_net, nl.num_nets, nl.num_mov, 100)
    rng = np.random.default_rng(seed)
    pos = (rng.random((nl.num_mov + 17, 2)) * [nl.width, nl.height]).astype(np.float32)
    g = gp_cuda()
    grad, out = g.wa(cu(pos), cu(cs.cell32), cu(cs.off), cu(cs.net_start), cu(cs.cell_start), cu(cs.cell_pin),
                     nl.num_mov, cu(np.array([gamma], np.float32)))
    wa, ograd, hpwl, oout, _ = O.wa_forward(pos, cs.cell32, cs.off, cs.net_start, nl.num_mov, gamma)
    return grad.cpu().numpy(), out.cpu().numpy(), ograd, oout


@pytest.mark.parametrize("gamma", [40.0, 4.0, 0.3])
def test_wa_matches_oracle(gamma):
    nl = synth.make_netlist(5000, 5300, window=100, macros=4, cover=0.1, fixed_pin_share=0.05, seed=3)
    grad, out, ograd, oout = _wa_case(nl, gamma)
    assert relerr(grad, ograd) <= 1e-5
    assert np.abs(out[:, 1] - oout[:, 1]).max() <= 1e-6 * np.abs(oout[:, 1]).max()      # HPWL: max / min
    assert np.abs(out[:, 0] - oout[:, 0]).max() <= 1e-5 * np.abs(oout[:, 0]).max()


def test_wa_golden(gold):
    g = gold("golden_wa.npz")
    n = int(g["num_mov"])
    grad, out = gp_cuda().wa(cu(g["pos"]), cu(g["cell32"]), cu(g["off_opt"]), cu(g["net_start"]), cu(g["cell_start"]),
                             cu(g["cell_pin"]), n, cu(np.array([g["gamma1"]], np.float32)))
    assert relerr(grad.cpu().numpy(), g["grad1"]) <= 1e-5
    tot = out.double().sum(0).cpu().numpy()
    assert abs(tot[0] - float(g["wa1"])) <= 1e-5 * abs(tot[0])
    assert abs(tot[1] - float(g["hpwl1"])) <= 1e-6 * tot[1]


def test_wa_empty_and_errors():
    g = gp_cuda()
    grad, out = g.wa(cu(np.zeros((3, 2), np.float32)), cu(np.zeros(0, np.int32)), cu(np.zeros((0, 2), np.float32)),
                     cu(np.zeros(1, np.int32)), cu(np.zeros(4, np.int32)), cu(np.zeros(0, np.int32)), 3,
                     cu(np.array([1.0], np.float32)))
    torch.cuda.synchronize()
    assert grad.shape == (3, 2) and float(grad.abs().sum()) == 0.0 and out.shape == (0, 2)
    with pytest.raises(RuntimeError, match="float32"):
        g.wa(cu(np.zeros((3, 2), np.float64)), cu(np.zeros(0, np.int32)), cu(np.zeros((0, 2), np.float32)),
             cu(np.zeros(1, np.int32)), cu(np.zeros(4, np.int32)), cu(np.zeros(0, np.int32)), 3,
             cu(np.array([1.0], np.float32)))


# ------------------------------------------------------------------------------------------------ density map
def _density_case(seed=1, cells=3000, nb=64, clump=True):
    nl = synth.make_netlist(cells, cells + 100, window=60, macros=3, cover=0.12, seed=seed)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=nb // 2, force_num_bin=nb))
    gr = prob.force
    rng = np.random.default_rng(seed)
    pos = (rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]).astype(np.float32)
    if clump:
        pos[:cells // 3] = pos[:cells // 3] * 0.01 + np.array([nl.width * 0.4, nl.height * 0.55], np.float32)
    pos = np.clip(pos, gr.pos_lo, gr.pos_hi).astype(np.float32)
    return prob, gr, pos


def _native_map(pos, size, ratio, num_mov, gr):
    m = torch.empty((2, gr.nbx, gr.nby), dtype=torch.int64, device=DEV)
    rho = torch.empty((2 * gr.nbx, 2 * gr.nby), device=DEV)
    over = torch.empty((gr.nbx, gr.nby), device=DEV)
    fixed = cu(gr.fixed_map)
    p, s, r = cu(pos), cu(size), cu(ratio)
    native.call("gp103_density_map", p.data_ptr(), s.data_ptr(), r.data_ptr(), len(pos), num_mov, gr.bx, gr.by,
                gr.nbx, gr.nby, m.data_ptr(), fixed.data_ptr(), gr.target, rho.data_ptr(), over.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return m.cpu().numpy().view(np.uint64), rho.cpu().numpy(), over.cpu().numpy()


@pytest.mark.parametrize("clump", [False, True])
def test_density_map_bit_exact(clump):
    prob, gr, pos = _density_case(clump=clump)
    m, rho, over = _native_map(pos, gr.size, gr.ratio, prob.num_mov, gr)
    om = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    assert np.array_equal(m, om)
    orho, oover, _ = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    assert np.array_equal(rho.view(np.uint32), orho.view(np.uint32))
    assert np.array_equal(over.view(np.uint32), oover.view(np.uint32))


def test_density_map_repeatable_and_drop_in():
    prob, gr, pos = _density_case(seed=5, cells=20000, nb=128)
    a = _native_map(pos, gr.size, gr.ratio, prob.num_mov, gr)
    b = _native_map(pos, gr.size, gr.ratio, prob.num_mov, gr)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    rho, over = gp_cuda().density_map(cu(pos), cu(gr.size), cu(gr.ratio), prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby,
                                      cu(gr.fixed_map), gr.target)
    assert np.array_equal(rho.cpu().numpy(), a[1]) and np.array_equal(over.cpu().numpy(), a[2])


def test_density_map_edge_cases():
    nb = 16
    nl = synth.make_netlist(200, 210, window=20, seed=2)
    prob = problem.Problem(nl, problem.options(num_bin=nb, force_num_bin=nb))
    gr = prob.force
    pos = np.clip(np.random.default_rng(0).random((prob.num_nodes, 2)) * [nl.width, nl.height], gr.pos_lo,
                  gr.pos_hi).astype(np.float32)
    # no nodes at all
    m, rho, over = _native_map(pos[:0], gr.size[:0], gr.ratio[:0], 0, gr)
    assert not m.any() and np.array_equal(over, np.maximum(gr.fixed_map - gr.target, 0))
    # nodes on the region's edges and corners, and one node over the whole region
    pos[0] = gr.pos_lo[0]
    pos[1] = gr.pos_hi[1]
    size = gr.size.copy()
    size[2] = [nl.width, nl.height]
    pos[2] = [nl.width / 2, nl.height / 2]
    m, _, _ = _native_map(pos, size, gr.ratio, prob.num_mov, gr)
    assert np.array_equal(m, O.density_map(pos, size, gr.ratio, prob.num_mov, gr.bx, gr.by, nb, nb))
    # a node that is not finite adds what the reference's kernel adds (float -> int conversions of the GPU)
    pos[3] = [np.nan, 5.0]
    pos[4] = [np.inf, -np.inf]
    m, _, _ = _native_map(pos, size, gr.ratio, prob.num_mov, gr)
    assert np.array_equal(m, O.density_map(pos, size, gr.ratio, prob.num_mov, gr.bx, gr.by, nb, nb))


# ------------------------------------------------------------------------------------------------ gather
def test_density_grad_matches_oracle():
    prob, gr, pos = _density_case(seed=7, cells=4000, nb=64)
    om = O.density_map(pos, gr.size, gr.ratio, prob.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
    orho, _, _ = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby)
    field = O.field_fft(orho, gr.nbx, gr.nby, gr.bin_np)
    rng = np.random.default_rng(1)
    wl = rng.standard_normal((prob.num_mov, 2)).astype(np.float32)
    for weight, precond in ((0.37, 0.37), (1.0, -1.0)):
        grad = gp_cuda().density_grad(cu(pos), cu(gr.size), cu(gr.ratio), cu(field.astype(np.float32)), cu(wl),
                                      cu(prob.pins), cu(prob.area), cu(np.array([weight], np.float32)),
                                      cu(np.array([precond], np.float32)), gr.bx, gr.by, gr.nbx, gr.nby)
        og = O.density_grad(pos, gr.size, gr.ratio, field[0], field[1], wl, prob.pins, prob.area, weight, precond,
                            gr.bx, gr.by, gr.nbx, gr.nby)
        assert relerr(grad.cpu().numpy(), og) <= 1e-5


# ------------------------------------------------------------------------------------------------ step, control
def test_nesterov_step_and_select():
    rng = np.random.default_rng(4)
    n = 10007
    u, v, g = (rng.standard_normal(n).astype(np.float32) * 100 for _ in range(3))
    lo, hi = np.full(n, -80, np.float32), np.full(n, 90, np.float32)
    un, vn = gp_cuda().nesterov_step(cu(u), cu(v), cu(g), cu(lo), cu(hi), cu(np.array([0.7], np.float32)),
                                     cu(np.array([0.3], np.float32)))
    ou, ov = O.nesterov_step(u, v, g, lo, hi, np.float32(0.7), np.float32(0.3))
    assert np.abs(un.cpu().numpy() - ou).max() <= 1e-4 and np.abs(vn.cpu().numpy() - ov).max() <= 1e-4
    S = np.zeros(21)
    for accept, best in ((0, 0), (1, 0), (1, 1)):
        S[O.K["accept"]], S[O.K["is_best"]] = accept, best
        t = [cu(x.copy()) for x in (u, v, g)] + [cu(np.zeros(n, np.float32))]
        gp_cuda().select(cu(S), t[0], t[1], t[2], un, vn, cu(g * 2), t[3])
        assert np.array_equal(t[1].cpu().numpy(), vn.cpu().numpy() if accept else v)
        assert np.array_equal(t[3].cpu().numpy(), vn.cpu().numpy() if best else np.zeros(n, np.float32))


@pytest.mark.parametrize("accuracy", [True, False])
def test_control_matches_oracle(gold, accuracy):
    from tests.test_oracle_golden import _control_state
    g = gold("golden_control.npz")
    rows = g["rows"][g["accuracy"] == accuracy]
    S, c = _control_state(g, accuracy)
    kp = np.zeros(5, np.float32)
    dS, dkp, dc = cu(S.copy()), cu(kp.copy()), cu(c)
    sc = lambda x: cu(np.array(x, np.float32).reshape(()))
    for r in rows:
        moved, hpwl, ovf, wa = (float(np.float32(x)) for x in (r[3], r[1], r[2], r[4]))
        O.control(S, kp, c, moved, 1.0, hpwl, ovf, wa)
        gp_cuda().control(dS, dkp, dc, sc(moved), sc(1.0), sc(hpwl), sc(ovf), sc(wa))
        got = dS.cpu().numpy()
        assert np.allclose(got, S, rtol=1e-12, atol=0, equal_nan=True), r[0]
        assert np.array_equal(dkp.cpu().numpy(), kp)


def test_control_divergence():
    S = np.zeros(21)
    S[O.K["gam"]] = S[O.K["a"]] = S[O.K["alpha"]] = 1.0
    S[O.K["best_hpwl"]] = S[O.K["best_ovf"]] = math.inf
    c = np.array([1.0, 10.0, 100.0, 100.0, 1.0, 0, 0.07, 3, 50, 1e9, 1.0, 1.0, 0.0])
    dS, dkp = cu(S), cu(np.zeros(5, np.float32))
    sc = lambda x: cu(np.array(x, np.float32).reshape(()))
    gp_cuda().control(dS, dkp, cu(c), sc(1.0), sc(float("nan")), sc(100.0), sc(0.5), sc(90.0))
    got = dS.cpu().numpy()
    assert got[O.K["stop"]] == 3 and got[O.K["accept"]] == 0


# ------------------------------------------------------------------------------------------------ field
def _field_plan(nb, mode, bx=7.3, by=6.1):
    """A minimal plan with only the field buffers filled (gp103_field needs no netlist); nb: n or (nbx, nby)."""
    nbx, nby = nb if isinstance(nb, tuple) else (nb, nb)
    s = native.Sizes()
    native.call("gp103_plan_sizes", nbx, nby, mode, ctypes.byref(s))
    keep = dict(c=torch.zeros(s.field_const, dtype=torch.uint8, device=DEV),
                w=torch.zeros(s.field_work, dtype=torch.uint8, device=DEV),
                red=torch.zeros(s.red, dtype=torch.float64, device=DEV),
                cnt=torch.zeros(16, dtype=torch.int32, device=DEV),
                map=torch.zeros((2, nbx, nby), dtype=torch.int64, device=DEV),
                ex=torch.zeros((nbx, nby), device=DEV), ey=torch.zeros((nbx, nby), device=DEV),
                kp=torch.zeros(5, device=DEV))
    pl = native.Plan()
    pl.nbx, pl.nby = nbx, nby
    pl.bx, pl.by = bx, by
    pl.field_mode = mode
    pl.field_const, pl.field_work = keep["c"].data_ptr(), keep["w"].data_ptr()
    pl.red, pl.counters, pl.map = keep["red"].data_ptr(), keep["cnt"].data_ptr(), keep["map"].data_ptr()
    pl.ex, pl.ey, pl.kp = keep["ex"].data_ptr(), keep["ey"].data_ptr(), keep["kp"].data_ptr()
    native.call("gp103_field_constants", ctypes.byref(pl), torch.cuda.current_stream().cuda_stream)
    return pl, keep


def _density_plane(nb, seed=0):
    nbx, nby = nb if isinstance(nb, tuple) else (nb, nb)
    rng = np.random.default_rng(seed)
    a = rng.random((nbx, nby)) * 0.3 + 0.6
    a[nbx // 3: nbx // 3 + 5, nby // 2: nby // 2 + 7] += 40.0      # a clump
    a[: nbx // 4, -nby // 5:] = 0.9                                 # a blocked corner
    return a.astype(np.float32)


@pytest.mark.parametrize("nb,mode,tol", [(64, native.FIELD_FP32, 2e-6), (128, native.FIELD_FP32, 2e-6),
                                         (128, native.FIELD_BF16X6, 1e-6), (256, native.FIELD_BF16X6, 1e-6),
                                         (256, native.FIELD_BF16X3, 3e-5), (128, native.FIELD_F16X3, 1e-6),
                                         (256, native.FIELD_F16X3, 1e-6), (1024, native.FIELD_F16X3, 1e-6),
                                         (1024, native.FIELD_BF16X6, 1e-6), ((256, 512), native.FIELD_F16X3, 1e-6),
                                         ((512, 256), native.FIELD_F16X3, 1e-6),
                                         ((256, 384), native.FIELD_F16X3, 1e-6), (128, native.FIELD_TF32X3, 1e-6),
                                         (256, native.FIELD_TF32X3, 1e-6), (1024, native.FIELD_TF32X3, 1e-6),
                                         ((256, 384), native.FIELD_TF32X3, 1e-6)])
def test_field_matches_fp64(nb, mode, tol):
    """The field against its float64 statement and the reference's mirrored FFT. f16x3 folds the transforms on grids
    whose sides are multiples of 256 (256, 1024, 256 x 512, 512 x 256: the x and y folds each on a grid where the
    other side differs), not on 128 or 256 x 384."""
    nbx, nby = nb if isinstance(nb, tuple) else (nb, nb)
    pl, keep = _field_plan(nb, mode)
    a = _density_plane(nb)
    ex, ey = torch.zeros((nbx, nby), device=DEV), torch.zeros((nbx, nby), device=DEV)
    d = cu(a)
    native.call("gp103_field", ctypes.byref(pl), d.data_ptr(), ex.data_ptr(), ey.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    fx, fy = O.field_dct(a, np.array([7.3, 6.1]))
    scale = max(np.abs(fx).max(), np.abs(fy).max())
    err = max(np.abs(ex.cpu().numpy() - fx).max(), np.abs(ey.cpu().numpy() - fy).max()) / scale
    assert err <= tol, err
    # the same as the first quadrant of the reference's mirrored FFT field
    f64 = O.field_fft(O.mirror(a), nbx, nby, np.array([7.3, 6.1]))
    assert np.abs(ex.cpu().numpy() - f64[0, :nbx, :nby]).max() <= 2 * tol * scale
