"""ORACLE — test infrastructure only: the per-step field precision of a placement run against float64.

For a placement of a netlist with a given field mode, every `every` density passes the current positions' density
map is taken (gp103_density_map: the run's own fixed-point map) and its field is computed three ways:
  - the mode under test (gp103_field with the Placer's plan: the same kernels and shift as the run's passes);
  - the reference's float32 formula: the FFT of the mirrored map times the spectral operator, complex64
    (src/core/electronic_density_layer.py:70-77,133), by torch.fft on the GPU -- the plain path of the comparison;
  - float64: the cosine / sine transforms of the map (torch float64 matrix products on the GPU), equal to the mirrored
    FFT field (tests/test_oracle_golden.py pins the formulas to each other).
Reported per step: max |E - E64| / max |E64| over both planes, and the relative error of the field energy
sum(Ex^2 + Ey^2) (the reference computes no potential; the energy is the potential's counterpart that the field
determines). Only tests/ and the c1 report use this module.
"""
import ctypes
import math

import numpy as np
import torch


def _dct64(n, dev):
    p = torch.arange(n, dtype=torch.float64, device=dev)[:, None]
    u = torch.arange(n, dtype=torch.float64, device=dev)[None, :]
    t = math.pi * p * (2 * u + 1) / (2 * n)
    return torch.cos(t), torch.sin(t)


class Fp64Field(object):
    """E = (Sx^T (C * Wx) Cy, Cx^T (C * Wy) Sy), C = Cx A Cy^T, in float64 on the GPU (the oracle's field_dct)."""

    def __init__(self, nbx, nby, bin_np, dev):
        self.cx, self.sx = _dct64(nbx, dev)
        self.cy, self.sy = _dct64(nby, dev)
        bx, by = float(bin_np[0]), float(bin_np[1])
        p = torch.arange(nbx, dtype=torch.float64, device=dev)[:, None]
        q = torch.arange(nby, dtype=torch.float64, device=dev)[None, :]
        kx, ky = math.pi * p / (nbx * bx), math.pi * q / (nby * by)
        k2 = kx ** 2 + ky ** 2
        inv = torch.where(k2 > 0, 1.0 / torch.where(k2 > 0, k2, torch.ones_like(k2)), torch.zeros_like(k2)) / bx
        wq = torch.where(q == 0, 1.0, 2.0)
        wp = torch.where(p == 0, 1.0, 2.0)
        s = 2.0 / (nbx * nby)
        self.wx, self.wy = s * wq * kx * inv, s * wp * ky * inv

    def __call__(self, a):
        c = self.cx @ a.double() @ self.cy.T
        return self.sx.T @ (c * self.wx) @ self.cy, self.cx.T @ (c * self.wy) @ self.sy


class Fp32FftField(object):
    """The reference's float32 CPU/GPU formula: rfft2 of the mirrored map, times -i k / |k|^2 / bin_x (Nyquist and DC
    zeroed), irfft2; the first quadrant."""

    def __init__(self, nbx, nby, bin_np, dev):
        kx = 2 * math.pi * torch.fft.fftfreq(2 * nbx, d=float(bin_np[0]), device=dev).unsqueeze(1)
        ky = 2 * math.pi * torch.fft.rfftfreq(2 * nby, d=float(bin_np[1]), device=dev).unsqueeze(0)
        inv = 1.0 / (kx ** 2 + ky ** 2).clamp(min=1e-30)
        inv[0, 0] = 0.0
        inv = inv / float(bin_np[0])
        kx[nbx, 0] = 0.0
        ky[0, nby] = 0.0
        self.op = torch.stack([-1j * kx * inv, -1j * ky * inv]).to(torch.complex64)
        self.nbx, self.nby = nbx, nby

    def __call__(self, a):
        m = torch.cat([a, a.flip(0)], 0)
        m = torch.cat([m, m.flip(1)], 1).float()
        f = torch.fft.irfft2(torch.fft.rfft2(m)[None] * self.op, s=(2 * self.nbx, 2 * self.nby))
        return f[0, :self.nbx, :self.nby], f[1, :self.nbx, :self.nby]


def errors(e, ref):
    """(max |E - E64| / max |E64|, |energy - energy64| / energy64) of a field (Ex, Ey) against float64."""
    ex, ey = (t.double() for t in e)
    rx, ry = ref
    scale = max(float(rx.abs().max()), float(ry.abs().max()), 1e-300)
    err = max(float((ex - rx).abs().max()), float((ey - ry).abs().max())) / scale
    en, en64 = float((ex * ex + ey * ey).sum()), float((rx * rx + ry * ry).sum())
    return err, abs(en - en64) / max(en64, 1e-300)


def density_plane(placer, pos):
    """The run's total density [nbx, nby] (float32) at pos: the fixed-point map of the force grid."""
    from autoplace_gb300 import native
    p, f, s = placer.p, placer.p.force, placer.stream
    with torch.cuda.stream(s):
        m = torch.empty((2, f.nbx, f.nby), dtype=torch.int64, device=placer.dev)
        rho = torch.empty((2 * f.nbx, 2 * f.nby), device=placer.dev)
        over = torch.empty((f.nbx, f.nby), device=placer.dev)
    native.call("gp103_density_map", pos.data_ptr(), placer.size.data_ptr(), placer.ratio.data_ptr(), p.num_nodes,
                p.num_mov, f.bx, f.by, f.nbx, f.nby, m.data_ptr(), placer.fixed.data_ptr(), f.target,
                rho.data_ptr(), over.data_ptr(), s.cuda_stream)
    return rho[:f.nbx, :f.nby].contiguous()


def field_of(placer, dens):
    """The field of a density with the Placer's own mode, plan and shift (gp103_field)."""
    from autoplace_gb300 import native
    f = placer.p.force
    with torch.cuda.stream(placer.stream):
        ex = torch.empty((f.nbx, f.nby), device=placer.dev)
        ey = torch.empty((f.nbx, f.nby), device=placer.dev)
    native.call("gp103_field", placer._ref, dens.data_ptr(), ex.data_ptr(), ey.data_ptr(), placer.stream.cuda_stream)
    return ex, ey


def run_with_errors(placer, pos0, every=8):
    """Place from pos0 (one level), eagerly, measuring the field error of every `every`-th density pass.
    -> (result of Placer.run, list of per-step dicts: pass, error of the mode, energy error, error of the FP32 FFT
    formula, its energy error)."""
    from autoplace_gb300 import native
    f = placer.p.force
    f64 = Fp64Field(f.nbx, f.nby, f.bin_np, placer.dev)
    fft = Fp32FftField(f.nbx, f.nby, f.bin_np, placer.dev)
    rows = []
    orig = placer._passes
    count = [0]

    def passes(phase, k, split=None):
        for _ in range(k):
            orig(phase, 1, split)
            if phase != native.PHASE_DENSITY:
                continue
            count[0] += 1
            if count[0] % every:
                continue
            with torch.cuda.stream(placer.stream):
                cur = int(placer.cur.cpu())
                d = density_plane(placer, placer.V[cur])
                ref = f64(d)
                e_m, en_m = errors(field_of(placer, d), ref)
                e_f, en_f = errors(fft(d), ref)
            rows.append({"pass": count[0], "mode_err": e_m, "mode_energy_err": en_m, "fft32_err": e_f,
                         "fft32_energy_err": en_f})

    placer._passes = passes
    placer.use_graphs = False
    try:
        r = placer.run(pos0)
    finally:
        placer._passes = orig
    return r, rows
