"""Drop-in replacement of AutoPlace's `gp_cuda` module (cpp_to_py/gp_cuda.cpp:78-85): the same six functions with
the same arguments, results and errors, computed by the sm_103a kernels of libgp103.so.

    from autoplace_gb300 import gp_cuda
    grad, out = gp_cuda.wa(pos, pin_cell, pin_off, net_start, cell_start, cell_pin, num_mov, gamma)

Every tensor must be a contiguous CUDA tensor of the stated dtype (float32, float64 for S / c, int32 for indices),
else RuntimeError, as the reference's TORCH_CHECKs (gp_cuda.cpp:16-28). Outputs are new tensors from torch's caching
allocator; control and select update their arguments in place. Kernels run on the current CUDA stream of the
tensors' device (the reference uses the legacy default stream); a failed launch raises RuntimeError."""
import torch

from . import native

__all__ = ["wa", "density_map", "nesterov_step", "density_grad", "control", "select"]


def _check(t, dtype, what):
    if not (torch.is_tensor(t) and t.is_cuda and t.is_contiguous() and t.dtype == dtype):
        raise RuntimeError("want a contiguous %s CUDA tensor" % what)
    return t.data_ptr()


def F(t):
    return _check(t, torch.float32, "float32")


def D(t):
    return _check(t, torch.float64, "float64")


def I(t):
    return _check(t, torch.int32, "int32")


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def wa(pos, pin_cell, pin_off, net_start, cell_start, cell_pin, num_mov, gamma):
    """-> (gradient [num_mov, 2], per-net (WA, HPWL) [num_nets, 2])."""
    num_nets = net_start.size(0) - 1
    args = (F(pos), I(pin_cell), F(pin_off), I(net_start), I(cell_start), I(cell_pin))
    gp = F(gamma)
    pin_grad = torch.empty_like(pin_off)
    out = pos.new_empty((num_nets, 2))
    grad = pos.new_empty((num_mov, 2))
    native.call("gp103_wa", *args, num_nets, num_mov, gp, pin_grad.data_ptr(), out.data_ptr(), grad.data_ptr(),
                _stream(pos))
    return grad, out


def density_map(pos, size, ratio, num_mov, bx, by, nbx, nby, fixed, target):
    """-> (total density mirrored [2 nbx, 2 nby], density of cells + blocked area above the target [nbx, nby])."""
    args = (F(pos), F(size), F(ratio))
    fx = F(fixed)
    m = torch.empty((2, nbx, nby), dtype=torch.int64, device=pos.device)
    rho = pos.new_empty((2 * nbx, 2 * nby))
    over = pos.new_empty((nbx, nby))
    native.call("gp103_density_map", *args, pos.size(0), num_mov, float(bx), float(by), nbx, nby, m.data_ptr(), fx,
                float(target), rho.data_ptr(), over.data_ptr(), _stream(pos))
    return rho, over


def nesterov_step(u, v, g, lo, hi, alpha, coef):
    """-> (u_next, v_next) of Nesterov's method; v_next kept inside [lo, hi]."""
    args = (F(u), F(v), F(g), F(lo), F(hi), F(alpha), F(coef))
    u_next, v_next = torch.empty_like(v), torch.empty_like(v)
    native.call("gp103_nesterov_step", *args, v.numel(), u_next.data_ptr(), v_next.data_ptr(), _stream(v))
    return u_next, v_next


def density_grad(pos, size, ratio, field, wl_grad, pins, area, weight, precond, bx, by, nbx, nby):
    """field [2, 2 nbx, 2 nby]; wl_grad [num_wl, 2] (num_wl may be 0) -> preconditioned gradient [num_nodes, 2]."""
    args = (F(pos), F(size), F(ratio), F(field), F(wl_grad), F(pins), F(area))
    w, p = F(weight), F(precond)
    grad = torch.empty_like(pos)
    native.call("gp103_density_grad", *args, pos.size(0), wl_grad.size(0), w, p, float(bx), float(by), nbx, nby,
                grad.data_ptr(), _stream(pos))
    return grad


def control(S, kp, c, moved, turned, hpwl, ovf, wa):
    """One pass of the run's control: S (float64 [21]) and kp (float32 [5]) updated in place."""
    args = (D(S), F(kp), D(c), F(moved), F(turned), F(hpwl), F(ovf), F(wa))
    native.call("gp103_control", *args, _stream(S))


def select(S, u, v, g, u_next, v_next, g_next, best):
    """Take the pass's step if it was accepted (u, v, g in place); copy it to best if it is the best so far."""
    args = (D(S), F(u), F(v), F(g), F(u_next), F(v_next), F(g_next), F(best))
    native.call("gp103_select", *args, v.numel(), _stream(v))
