"""The drop-in driven the way the reference drives its own `gp_cuda` module: one level of global placement written as
the reference's code runs it with the CUDA extension loaded, every kernel call going through
`autoplace_gb300.gp_cuda` (the shim that replaces the reference's extension), against the reference's own run of the
same level (golden_place.npz, recorded from the reference itself).

The reference's sources are not available where this test runs, so its loop is restated here, call for call:
  - `_place_level` (src/run_placement.py:41-76): the initial step length, the optimiser, the wirelength-only start
    until ParamScheduler.start_step ends it, the density weight in tension units, then `run_level_on_gpu`;
  - NesterovOptimizer (src/nesterov_optimizer.py:15-61) with `gp_cuda.nesterov_step`;
  - Objective.__call__ / on_gpu / tension_unit (src/calculator.py:20-43);
  - Wirelength.forward with `gp_cuda.wa` (src/core/wa_wirelength_hpwl.py:90-97);
  - ElectronicDensityLayer.forward with `gp_cuda.density_map` and `gp_cuda.density_grad`, the field by torch's FFT of
    the mirrored map (src/core/electronic_density_layer.py:70-77,96-149), the overflow on the overflow grid;
  - run_level_on_gpu (src/gpu_loop.py:35-81) with `gp_cuda.control` and `gp_cuda.select`, the host looking every 16
    passes.
The bars are those of the GPU engine's own comparison with the same run: the same stop reason and wirelength-only
start, iterations within 5 %, exact HPWL within 0.5 %."""
import math
from types import SimpleNamespace

import numpy as np
import pytest

from autoplace_gb300 import problem, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"
FIELDS = ("lam gam alpha a iter hpwl_prev motion ww mu settled best_hpwl best_ovf is_best improved stop accept "
          "loop_it evals res_hpwl res_ovf has_best").split()
K = {name: i for i, name in enumerate(FIELDS)}
REASON = {1: "converged", 2: "stalled", 3: "diverged", 4: "max_iter", 5: "handover"}


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(dtype=dt, device=DEV).contiguous()


class Density(object):
    """ElectronicDensityLayer's kernel path on one grid of the problem (`grid`: prob.force or prob.judge)."""

    def __init__(self, prob, grid, field=True):
        self.g, self.n = grid, prob.num_mov
        self.size, self.ratio = _t(grid.size), _t(grid.ratio)
        self.fixed = _t(grid.fixed_map)
        self.pins, self.area = _t(prob.pins), _t(prob.area)
        self.no_grad = torch.zeros(0, 2, device=DEV)
        self.scal = torch.empty(2, device=DEV)
        self.judge = None
        if field:                                   # the reference's operator of the mirrored map's spectrum
            nbx, nby, bx, by = grid.nbx, grid.nby, grid.bx, grid.by
            kx = 2 * math.pi * torch.fft.fftfreq(2 * nbx, d=bx).to(DEV).unsqueeze(1)
            ky = 2 * math.pi * torch.fft.rfftfreq(2 * nby, d=by).to(DEV).unsqueeze(0)
            inv = 1.0 / (kx ** 2 + ky ** 2).clamp_(min=1e-30)
            inv[0, 0] = 0.0
            inv = inv / bx
            kx[nbx, 0] = 0.0
            ky[0, nby] = 0.0
            self.to_field = torch.stack([-1j * kx * inv, -1j * ky * inv]).to(torch.complex64)

    def _density(self, pos):
        g = self.g
        rho, over = gp_cuda().density_map(pos, self.size, self.ratio, self.n, g.bx, g.by, g.nbx, g.nby, self.fixed,
                                          g.target)
        return rho, over.sum() * (g.bin_area / g.mov_area)

    def smoothed_overflow(self, pos):
        return self._density(pos[:self.n].contiguous())[1]

    def forward(self, pos, wl_grad=None, weight=1.0, precond=-1.0):
        g = self.g
        rho, overflow = self._density(pos)
        if self.judge is not None:
            overflow = self.judge.smoothed_overflow(pos)
        field = torch.fft.irfft2(torch.fft.rfft2(rho) * self.to_field, s=(2 * g.nbx, 2 * g.nby)).contiguous()
        wl_grad = self.no_grad if wl_grad is None else wl_grad
        if not torch.is_tensor(weight):
            weight = self.scal[0:1].fill_(weight)
        if not torch.is_tensor(precond):
            precond = self.scal[1:2].fill_(precond)
        grad = gp_cuda().density_grad(pos, self.size, self.ratio, field, wl_grad, self.pins, self.area, weight,
                                      precond, g.bx, g.by, g.nbx, g.nby)
        return grad, overflow


class Wirelength(object):
    def __init__(self, prob):
        cs = prob.csr
        self.cell32, self.off, self.net_start = _t(cs.cell32, torch.int32), _t(cs.off), _t(cs.net_start, torch.int32)
        self.cell_start, self.cell_pin = _t(cs.cell_start, torch.int32), _t(cs.cell_pin, torch.int32)
        self.n = prob.num_mov
        self.gamma = torch.empty(1, device=DEV)

    def forward(self, pos, gamma):
        if not torch.is_tensor(gamma):
            gamma = self.gamma.fill_(gamma)
        grad, out = gp_cuda().wa(pos, self.cell32, self.off, self.net_start, self.cell_start, self.cell_pin, self.n,
                                 gamma)
        total = out.sum(0)
        return total[0], grad, total[1]


class Objective(object):
    def __init__(self, wl, density, ps):
        self.wl, self.density, self.ps = wl, density, ps
        self.wa = self.hpwl = self.overflow = None
        self.evals = 0
        self.not_measured = torch.tensor(float("nan"), device=DEV)
        self.pin_precond = density.pins[:density.n].clamp(min=1.0).unsqueeze(1)

    def tension_unit(self, pos):
        n = self.density.n
        return (self.density.pins.sum() / self.density.forward(pos)[0][:n].abs().sum()).item()

    def __call__(self, pos):
        self.wa, wl_grad, self.hpwl = self.wl.forward(pos, self.ps.wa_coeff)
        if self.ps.density_weight == 0:
            grad, self.overflow = torch.zeros_like(pos), self.not_measured
            grad[:len(wl_grad)] = wl_grad / self.pin_precond
        else:
            grad, self.overflow = self.density.forward(pos, wl_grad, self.ps.density_weight, self.ps.density_weight)
        self.evals += 1
        return grad

    def on_gpu(self, pos, kp):
        self.wa, wl_grad, self.hpwl = self.wl.forward(pos, kp[0:1])
        grad, self.overflow = self.density.forward(pos, wl_grad, kp[1:2], kp[2:3])
        self.evals += 1
        return grad


class Nesterov(object):
    def __init__(self, pos, grad_fn, lr, lo, hi, stats):
        self.grad_fn, self.stats, self.lo, self.hi = grad_fn, stats, lo, hi
        self.scal = pos.new_empty(2)
        self.v = torch.max(torch.min(pos, hi), lo)
        self.g = grad_fn(self.v)
        self.u = self.v.clone()
        probe = torch.max(torch.min(torch.add(self.v, self.g, alpha=-lr), hi), lo)
        self.alpha = (torch.dist(self.v, probe) / torch.dist(self.g, grad_fn(probe))).item()
        self.a, self.moved, self.diverged, self.fetched = 1.0, 0.0, False, []

    def step(self):
        a_next = (1 + math.sqrt(4 * self.a * self.a + 1)) / 2
        coef = (self.a - 1) / a_next
        u_next, v_next = gp_cuda().nesterov_step(self.u, self.v, self.g, self.lo, self.hi,
                                                 self.scal[0:1].fill_(self.alpha), self.scal[1:2].fill_(coef))
        g_next = self.grad_fn(v_next)
        moved, turned, *self.fetched = torch.stack(
            (torch.dist(v_next, self.v), torch.dist(g_next, self.g)) + tuple(self.stats())).tolist()
        if not all(map(math.isfinite, [moved, turned] + self.fetched[:1])):
            self.diverged = True
            return
        self.moved = moved
        self.alpha = moved / turned if turned > 0 else self.alpha
        self.u, self.g, self.a = u_next, g_next, a_next
        self.v.copy_(v_next)


def gp_cuda():
    from autoplace_gb300 import gp_cuda as shim
    return shim


def _next_coef(a):
    a_next = (1 + math.sqrt(4 * a * a + 1)) / 2
    return (a - 1) / a_next


def run_level_on_gpu(opt, obj, ps, prob, iteration, check_every=16):
    """src/gpu_loop.py:35-81 with the shim's kernels."""
    o, sh = prob.opts, gp_cuda()
    pos = opt.v
    S = [0.0] * len(FIELDS)
    S[K["lam"]], S[K["gam"]], S[K["alpha"]], S[K["a"]] = ps.density_weight, ps.wa_coeff, opt.alpha, opt.a
    S[K["iter"]], S[K["hpwl_prev"]], S[K["motion"]], S[K["ww"]] = ps.iter, ps.hpwl[-1], 0.0, 0.0
    S[K["mu"]], S[K["settled"]], S[K["improved"]] = 1.0, 0, 0
    S[K["best_hpwl"]] = S[K["best_ovf"]] = float("inf")
    S[K["loop_it"]] = iteration
    S = torch.tensor(S, dtype=torch.float64, device=DEV)
    kp = torch.tensor([ps.wa_coeff, ps.density_weight, ps.density_weight, opt.alpha, _next_coef(opt.a)],
                      dtype=torch.float32, device=DEV)
    c = torch.tensor(prob.constants(), dtype=torch.float64, device=DEV)
    u, g, lo, hi = opt.u, opt.g, opt.lo, opt.hi
    best = pos.clone()
    watch = torch.tensor([K["stop"], K["loop_it"]], device=DEV)
    while True:
        for _ in range(check_every):
            u_next, v_next = sh.nesterov_step(u, pos, g, lo, hi, kp[3:4], kp[4:5])
            g_next = obj.on_gpu(v_next, kp)
            sh.control(S, kp, c, torch.dist(v_next, pos), torch.dist(g_next, g), obj.hpwl, obj.overflow, obj.wa)
            sh.select(S, u, pos, g, u_next, v_next, g_next, best)
        stop, it = S[watch].tolist()
        if stop:
            break
    S = S.tolist()
    if S[K["has_best"]]:
        pos.copy_(best)
    return REASON[int(S[K["stop"]])], int(S[K["loop_it"]])


def place_level(prob, pos0):
    """src/run_placement.py:41-76 (one level, from the first iteration), -> (reason, iterations, start iterations,
    final positions)."""
    o = prob.opts
    ps = SimpleNamespace(density_weight=0.0, wa_coeff=10 * prob.base_gamma, iter=0, hpwl=[], wa=[])
    density = Density(prob, prob.force)
    if prob.judge is not None:
        density.judge = Density(prob, prob.judge, field=False)
    obj = Objective(Wirelength(prob), density, ps)
    lo, hi = _t(prob.force.pos_lo), _t(prob.force.pos_hi)
    pos = _t(pos0)
    # estimate_initial_learning_rate (src/nesterov_optimizer.py:56-61)
    pos = torch.max(torch.min(pos, hi), lo)
    g = obj(pos)
    probe = torch.max(torch.min(pos - o.lr * g, hi), lo)
    lr = ((pos - probe).norm() / (g - obj(probe)).norm()).item()
    opt = Nesterov(pos, obj, lr, lo, hi, stats=lambda: (obj.hpwl, obj.overflow, obj.wa))
    start_iters = 0
    for iteration in range(0, int(o.inner_iter)):
        if ps.density_weight > 0:
            reason, iters = run_level_on_gpu(opt, obj, ps, prob, iteration)
            return reason, iters, start_iters, opt.v
        opt.step()
        assert not opt.diverged
        hpwl, overflow, wa = opt.fetched
        # ParamScheduler.start_step (src/param_scheduler.py:42-48), window 5
        ps.hpwl.append(hpwl)
        ps.wa.append(wa)
        ps.iter += 1
        w = 5
        if not (len(ps.wa) <= w or ps.wa[-1 - w] - wa > o.start_tol * w * wa):
            ps.density_weight, start_iters = o.density_weight * obj.tension_unit(opt.v), iteration + 1
    raise AssertionError("the wirelength-only start did not end")


def test_reference_loop_through_the_shim_matches_reference_run(gold):
    g = gold("golden_place.npz")
    nl = synth.make_netlist(int(g["cells"]), int(g["nets"]), window=int(g["window"]), macros=0, seed=int(g["seed"]))
    prob = problem.Problem(nl, problem.options(target_density=1.0, num_bin=int(g["num_bin"]), inner_iter=3000))
    reason, iters, start_iters, pos = place_level(prob, g["pos0"])
    torch.cuda.synchronize()
    h = O.hpwl_all(pos.cpu().numpy(), prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    print("shim-driven level: %s after %d iterations (start %d), hpwl %.6e; reference: %s, %d (start %d), %.6e"
          % (reason, iters, start_iters, h, str(g["reason"]), int(g["iters"]), int(g["start_iters"]),
             float(g["hpwl"])))
    assert reason == str(g["reason"])
    assert start_iters == int(g["start_iters"])
    assert abs(iters - int(g["iters"])) <= 0.05 * int(g["iters"])
    assert abs(h - float(g["hpwl"])) <= 0.005 * float(g["hpwl"])
