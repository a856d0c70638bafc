"""ORACLE — test infrastructure only.

CPU restatement of AutoPlace's global-placement iteration (the `gp_cuda` operators and the loop around them). Only
tests/, `__graft_entry__.smoke()` and the CPU-baseline leg of bench.py import this module, and only as the checker
or as the timed CPU baseline: the product (autoplace_gb300) never calls it.

Each function names the reference lines it restates (paths inside the AutoPlace project):

  build CSR       src/core/wa_wirelength_hpwl.py:26-44           (host numpy, shared with the product set-up)
  wa_forward      src/core/wa_wirelength_hpwl.py:83-94, gp_cuda_kernel.cu:12-57   float64
  hpwl_all        src/core/wa_wirelength_hpwl.py:66-70            float64
  density_map     gp_cuda_kernel.cu:71-95      C library, float32 op order of the kernel: the same integer map
  density_post    gp_cuda_kernel.cu:130-139    C library
  field_fft       src/core/electronic_density_layer.py:70-77,133  float64 (numpy pocketfft)
  field_dct       the same field as cosine/sine transforms of the plain [nbx, nby] map (float64)
  density_grad    gp_cuda_kernel.cu:102-125    C library, float64 accumulation
  nesterov_step   gp_cuda_kernel.cu:157-165, src/nesterov_optimizer.py:41-42
  control         gp_cuda_kernel.cu:183-240 with src/param_scheduler.py:63-116, src/resolution.py:33-56 (float64)
  select          gp_cuda_kernel.cu:243-249
  place_level     src/run_placement.py:41-76 + src/gpu_loop.py:35-81 (host loop; the CPU baseline)
  *_mt            multi-threaded forms (oracle/level_ref.c, OpenMP) of WA (float32), the map and the gather, for
                  CpuLevel(threads=...): a whole level of a large netlist on the host cores in minutes
  cluster_*       src/cluster.py:38-85 (star matching: pair edges, rounds), integer sums: exact
  coarse_pins     src/cluster.py:101-115 (the pins of the cluster problem)
  expand          src/cluster.py:133-144
  two_level       src/run_placement.py:87-110 with src/param_scheduler.py:53-60 (clusters first, then the cells)
"""
import ctypes
import math
import os
import subprocess
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
DENSITY_SCALE = 4294967296.0

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def lib():
    """The C restatement (oracle/density_ref.c), built on first use with oracle/Makefile."""
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        srcs = [os.path.join(_HERE, f) for f in ("density_ref.c", "level_ref.c", "Makefile")]
        if not os.path.exists(path) or os.path.getmtime(path) < max(os.path.getmtime(f) for f in srcs):
            subprocess.check_call(["make", "-s", "-C", _HERE])
        L = ctypes.CDLL(path)
        i, f, d = ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.oracle_density_map.argtypes = [_f32p, _f32p, _f32p, i, i, f, f, i, i, _u64p]
        L.oracle_density_map.restype = None
        L.oracle_density_post.argtypes = [_u64p, _f32p, f, i, i, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_density_post.restype = d
        L.oracle_density_grad.argtypes = [_f32p, _f32p, _f32p, _f64p, _f64p, i, ctypes.c_void_p, i, _f32p, _f32p, i,
                                          d, d, f, f, i, i, _f64p]
        L.oracle_density_grad.restype = None
        L.oracle_threads.argtypes = [i]
        L.oracle_threads.restype = i
        _i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.oracle_wa_mt.argtypes = [_f32p, _i32p, _f32p, _i32p, i, i, f, _i32p, _i32p, _f32p, _f32p, _f32p, _f64p]
        L.oracle_wa_mt.restype = None
        L.oracle_density_map_mt.argtypes = L.oracle_density_map.argtypes
        L.oracle_density_map_mt.restype = None
        L.oracle_density_grad_mt.argtypes = L.oracle_density_grad.argtypes
        L.oracle_density_grad_mt.restype = None
        _LIB = L
    return _LIB


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ------------------------------------------------------------------------------------------------ wirelength
def wa_forward(pos, cell32, off, net_start, num_mov, gamma, dtype=np.float64):
    """-> (WA total, grad [num_mov, 2], HPWL total, out [nets, 2] = per-net (WA, HPWL), pin gradient [P, 2]).

    Per net and axis: max / min, max-shifted exponent sums, WA = xp - xn, pin gradient
    ep (1 + (x - xp) / g) / sp - en (1 - (x - xn) / g) / sn; per cell the sum of its pins."""
    num_nets = len(net_start) - 1
    P = len(cell32)
    pos = np.asarray(pos, dtype=dtype)
    ext = np.concatenate([pos[:num_mov], np.zeros((1, 2), dtype)])
    x = ext[cell32] + np.asarray(off, dtype=dtype)
    if num_nets == 0:
        return 0.0, np.zeros((num_mov, 2), dtype), 0.0, np.zeros((0, 2), dtype), np.zeros((P, 2), dtype)
    starts = np.asarray(net_start[:-1], dtype=np.int64)
    net = np.repeat(np.arange(num_nets), np.diff(net_start))
    hi = np.maximum.reduceat(x, starts, axis=0)
    lo = np.minimum.reduceat(x, starts, axis=0)
    g = dtype(gamma)
    ep = np.exp((x - hi[net]) / g)
    en = np.exp((lo[net] - x) / g)
    sp = np.add.reduceat(ep, starts, axis=0)
    sn = np.add.reduceat(en, starts, axis=0)
    xp = np.add.reduceat(x * ep, starts, axis=0) / sp
    xn = np.add.reduceat(x * en, starts, axis=0) / sn
    gp = ep * (1 + (x - xp[net]) / g) / sp[net] - en * (1 - (x - xn[net]) / g) / sn[net]
    grad = np.stack([np.bincount(cell32, weights=gp[:, a], minlength=num_mov + 1)[:num_mov] for a in range(2)], 1)
    out = np.stack([(xp - xn).sum(1), (hi - lo).sum(1)], 1)
    return float(out[:, 0].sum()), grad.astype(dtype), float(out[:, 1].sum()), out, gp


def set_threads(n):
    """Threads of the multi-threaded oracle operators (0: leave as is) -> the count in force."""
    return int(lib().oracle_threads(int(n)))


def wa_forward_mt(pos, cell32, off, net_start, cell_start, cell_pin, num_mov, gamma):
    """wa_forward(dtype=float32) on the host threads (oracle/level_ref.c): the same arithmetic, each cell's pins summed
    in pin order. -> (WA total, grad [num_mov, 2] float32, HPWL total, out [nets, 2] float32, pin gradient [P, 2])."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    num_nets, P = len(net_start) - 1, len(cell32)
    pin_grad = np.empty((max(P, 1), 2), np.float32)
    grad = np.empty((max(num_mov, 1), 2), np.float32)
    out = np.empty((max(num_nets, 1), 2), np.float32)
    tot = np.zeros(2)
    lib().oracle_wa_mt(_c32(pos), i32(cell32), _c32(off), i32(net_start), num_nets, num_mov, float(gamma),
                       i32(cell_start), i32(cell_pin), pin_grad, grad, out, tot)
    return float(tot[0]), grad[:num_mov], float(tot[1]), out[:num_nets], pin_grad[:P]


def density_map_mt(pos, size, ratio, num_mov, bx, by, nbx, nby):
    """density_map on the host threads: the same integer map."""
    m = np.zeros((2, nbx, nby), dtype=np.uint64)
    lib().oracle_density_map_mt(_c32(pos), _c32(size), _c32(ratio), len(pos), num_mov, bx, by, nbx, nby, m)
    return m


def density_grad_mt(pos, size, ratio, fx, fy, wl_grad, pins, area, weight, precond, bx, by, nbx, nby):
    """density_grad on the host threads: the same values."""
    fx = np.ascontiguousarray(fx, np.float64)
    fy = np.ascontiguousarray(fy, np.float64)
    n = len(pos)
    wl = _c32(wl_grad) if wl_grad is not None and len(wl_grad) else None
    g = np.empty((n, 2), np.float64)
    lib().oracle_density_grad_mt(_c32(pos), _c32(size), _c32(ratio), fx, fy, fx.shape[1],
                                 wl.ctypes.data if wl is not None else None, 0 if wl is None else len(wl),
                                 _c32(pins), _c32(area), n, float(weight), float(precond), bx, by, nbx, nby, g)
    return g


def hpwl_all(pos, pin_cell, pin_off, net_start, num_mov):
    """Exact HPWL over every net (float64)."""
    pos = np.asarray(pos, dtype=np.float64)
    ext = np.concatenate([pos[:num_mov], np.zeros((1, 2))])
    x = ext[pin_cell] + np.asarray(pin_off, dtype=np.float64)
    deg = np.diff(net_start)
    starts = np.asarray(net_start[:-1], dtype=np.int64)[deg > 0]
    if len(starts) == 0:
        return 0.0
    return float((np.maximum.reduceat(x, starts, axis=0) - np.minimum.reduceat(x, starts, axis=0)).sum())


# ------------------------------------------------------------------------------------------------ density
def density_map(pos, size, ratio, num_mov, bx, by, nbx, nby):
    """-> the fixed-point map, uint64 [2, nbx, nby] (map 0: nodes below num_mov; map 1: the rest)."""
    m = np.zeros((2, nbx, nby), dtype=np.uint64)
    pos, size, ratio = _c32(pos), _c32(size), _c32(ratio)
    lib().oracle_density_map(pos, size, ratio, len(pos), num_mov, bx, by, nbx, nby, m)
    return m


def density_post(map_, fixed, target, nbx, nby, mirrored=True):
    """-> (rho mirrored [2 nbx, 2 nby] float32 or None, over [nbx, nby] float32, sum of over in float64)."""
    over = np.empty((nbx, nby), np.float32)
    rho = np.empty((2 * nbx, 2 * nby), np.float32) if mirrored else None
    total = lib().oracle_density_post(np.ascontiguousarray(map_, dtype=np.uint64), _c32(fixed), target, nbx, nby,
                                      rho.ctypes.data if mirrored else None, over.ctypes.data)
    return rho, over, total


def plain_density(map_, fixed):
    """Total density [nbx, nby] in float64 from the fixed-point map (the unmirrored rho)."""
    return map_[0].astype(np.float64) / DENSITY_SCALE + np.asarray(fixed, np.float64) + map_[1].astype(np.float64) / DENSITY_SCALE


def spectral_operator(nbx, nby, bin_np, dtype=np.float64):
    """The `to_field` operator of the mirrored map, [2, 2 nbx, nby + 1] complex."""
    kx = 2 * math.pi * np.fft.fftfreq(2 * nbx, d=float(bin_np[0])).astype(dtype)[:, None]
    ky = 2 * math.pi * np.fft.rfftfreq(2 * nby, d=float(bin_np[1])).astype(dtype)[None, :]
    inv = 1.0 / np.maximum(kx ** 2 + ky ** 2, dtype(1e-30))
    inv[0, 0] = 0.0
    inv = inv / dtype(bin_np[0])
    kx = kx.copy(); ky = ky.copy()
    kx[nbx, 0] = 0.0
    ky[0, nby] = 0.0
    return np.stack([-1j * kx * inv, -1j * ky * inv])


_OPS = {}


def field_fft(rho_mirrored, nbx, nby, bin_np, dtype=np.float64, workers=None):
    """Field of the mirrored map -> [2, 2 nbx, 2 nby] (x plane, y plane); float64, or float32 / complex64 as the
    reference's CPU path computes it. workers: transforms on that many host threads (scipy.fft), else numpy's."""
    key = (nbx, nby, float(bin_np[0]), float(bin_np[1]), np.dtype(dtype).name)
    op = _OPS.get(key)
    if op is None:
        op = spectral_operator(nbx, nby, bin_np)
        if dtype == np.float32:
            op = op.astype(np.complex64)
        _OPS.clear()
        _OPS[key] = op
    if workers:
        import scipy.fft as sf
        spec = sf.rfft2(np.asarray(rho_mirrored, dtype), workers=workers)
        return sf.irfft2(spec[None] * op, s=(2 * nbx, 2 * nby), workers=workers)
    spec = np.fft.rfft2(np.asarray(rho_mirrored, dtype))
    return np.fft.irfft2(spec[None] * op, s=(2 * nbx, 2 * nby))


def mirror(a):
    """[nbx, nby] -> the mirrored [2 nbx, 2 nby] map."""
    a = np.asarray(a)
    a = np.concatenate([a, a[::-1]], 0)
    return np.concatenate([a, a[:, ::-1]], 1)


def dct_matrices(n):
    """C[p, u] = cos(pi p (2u + 1) / 2n), S[p, u] = sin(pi p (2u + 1) / 2n), float64."""
    p = np.arange(n)[:, None]
    u = np.arange(n)[None, :]
    t = np.pi * p * (2 * u + 1) / (2 * n)
    return np.cos(t), np.sin(t)


def dct_weights(nbx, nby, bin_np):
    """Per-coefficient weights (Wx, Wy) [nbx, nby] of the field from the cosine coefficients: the mirrored-FFT
    operator folded onto the first quadrant (frequencies 0 .. n - 1 of each axis)."""
    bx, by = float(bin_np[0]), float(bin_np[1])
    p = np.arange(nbx)[:, None].astype(np.float64)
    q = np.arange(nby)[None, :].astype(np.float64)
    kx = math.pi * p / (nbx * bx)
    ky = math.pi * q / (nby * by)
    k2 = kx ** 2 + ky ** 2
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0) / bx
    wq = np.where(q == 0, 1.0, 2.0)
    wp = np.where(p == 0, 1.0, 2.0)
    scale = 2.0 / (nbx * nby)
    return scale * wq * kx * inv, scale * wp * ky * inv


def field_dct(density, bin_np):
    """Field of the plain map [nbx, nby] as cosine / sine transforms (float64) -> (Ex, Ey) [nbx, nby], equal to the
    first quadrant of `field_fft(mirror(density))`:
        C = Cx A Cy^T,  Ex = Sx^T (C * Wx) Cy,  Ey = Cx^T (C * Wy) Sy."""
    a = np.asarray(density, np.float64)
    nbx, nby = a.shape
    cx, sx = dct_matrices(nbx)
    cy, sy = dct_matrices(nby)
    wx, wy = dct_weights(nbx, nby, bin_np)
    c = cx @ a @ cy.T
    return sx.T @ (c * wx) @ cy, cx.T @ (c * wy) @ sy


def density_grad(pos, size, ratio, fx, fy, wl_grad, pins, area, weight, precond, bx, by, nbx, nby):
    """float64 gradient [n, 2]; fx / fy: planes [nbx, >= nby] (row stride = their second dimension)."""
    fx = np.ascontiguousarray(fx, np.float64)
    fy = np.ascontiguousarray(fy, np.float64)
    n = len(pos)
    wl = _c32(wl_grad) if wl_grad is not None and len(wl_grad) else None
    g = np.empty((n, 2), np.float64)
    lib().oracle_density_grad(_c32(pos), _c32(size), _c32(ratio), fx, fy, fx.shape[1],
                              wl.ctypes.data if wl is not None else None, 0 if wl is None else len(wl),
                              _c32(pins), _c32(area), n, float(weight), float(precond), bx, by, nbx, nby, g)
    return g


# ------------------------------------------------------------------------------------------------ clustering
def cluster_edges(pin_cell, pin_net, n, max_degree=8):
    """The pair edges of cluster_cells (src/cluster.py:44-56): for every net of at most max_degree pins (its degree
    counts every pin) each ordered pair of distinct movable cells (index < n) weighs 420 // (degree - 1), once per
    pair of its pins; the same (i, j) summed. -> (i, j, w) int64, sorted by i then j."""
    pin_cell = np.asarray(pin_cell, np.int64)
    pin_net = np.asarray(pin_net, np.int64)
    degree = np.bincount(pin_net)[pin_net]
    small = degree <= max_degree
    pc, pn, dg = pin_cell[small], pin_net[small], degree[small]
    keys, weights = [], []
    for k in range(1, max_degree):
        a, b, d = pc[:-k], pc[k:], dg[:-k]
        m = (pn[:-k] == pn[k:]) & (a < n) & (b < n) & (a != b)
        a, b, w = a[m], b[m], 420 // (d[m] - 1)
        keys += [a * n + b, b * n + a]
        weights += [w, w]
    if not keys:
        e = np.zeros(0, np.int64)
        return e, e, e
    key, inv = np.unique(np.concatenate(keys), return_inverse=True)
    w = np.zeros(len(key), np.int64)
    np.add.at(w, inv, np.concatenate(weights))
    return key // n, key % n, w


def cluster_round(i, j, w, area, head, cap, big, per_head=3):
    """One round of star matching (src/cluster.py:66-84). head [num] bool. A cluster that is not a head joins the head
    with the largest w / (area_i + area_j) among its edges (first such edge on ties), if the merged area is at most
    cap and neither is at or above big; a head takes the per_head largest scores (lower cluster index first on ties).
    -> (new index of every cluster, cluster areas, merged edges) or None when nothing merges."""
    num = len(area)
    total = area[i] + area[j]
    m = ~head[i] & head[j] & (total <= cap) & (area[i] < big) & (area[j] < big)
    tail, to, score = i[m], j[m], w[m].astype(np.float64) / total[m].astype(np.float64)
    # per tail: the best score, the first candidate (in edge order) on ties
    order = np.lexsort((np.arange(len(tail)), -score, tail))
    first = np.ones(len(order), bool)
    first[1:] = tail[order][1:] != tail[order][:-1]
    best = order[first]                                  # one per tail, tails ascending
    tail, to, score = tail[best], to[best], score[best]
    # per head: the per_head best scores, lower tail first on ties
    order = np.lexsort((tail, -score, to))
    g = to[order]
    start = np.ones(len(order), bool)
    start[1:] = g[1:] != g[:-1]
    pos = np.arange(len(order))
    rank = pos - np.maximum.accumulate(np.where(start, pos, 0))
    taken = order[rank < per_head]
    parent = np.arange(num)
    parent[tail[taken]] = to[taken]
    kept, new = np.unique(parent, return_inverse=True)
    if len(kept) == num:
        return None
    carea = np.zeros(len(kept), np.int64)
    np.add.at(carea, new, area)
    ni, nj = new[i], new[j]
    keep = ni != nj
    key, inv = np.unique(ni[keep] * len(kept) + nj[keep], return_inverse=True)
    nw = np.zeros(len(key), np.int64)
    np.add.at(nw, inv, w[keep])
    return new, carea, (key // len(kept), key % len(kept), nw)


def cluster_limits(area, ratio):
    """big and cap of cluster_cells (src/cluster.py:59-60) with the reference's own scalar arithmetic: torch on the
    CPU (a float ratio makes cap a float32 floor division)."""
    import torch
    a = torch.as_tensor(np.asarray(area, np.int64))
    big = 20 * a.sum() // len(a)
    small = a < big
    cap = 3 * ratio * a[small].sum() // (2 * int(small.sum()))
    return int(big), int(math.floor(float(cap)))


def cluster_cells(pin_cell, pin_net, area, ratio, draws, max_degree=8, per_head=3, max_rounds=12):
    """cluster_cells (src/cluster.py:38-85) with the head draws given: draws(r, num) -> float32 [num] uniform draws of
    round r (the reference's torch.rand of its seeded generator). -> (cluster of every cell, cluster areas)."""
    area = np.asarray(area, np.int64)
    n = len(area)
    i, j, w = cluster_edges(pin_cell, pin_net, n, max_degree)
    cid, num = np.arange(n), n
    big, cap = cluster_limits(area, ratio)
    for r in range(max_rounds):
        if num * ratio <= n:
            break
        head = np.asarray(draws(r, num)) < np.float32(0.5)
        res = cluster_round(i, j, w, area, head, cap, big, per_head)
        if res is None:
            break
        new, area, (i, j, w) = res
        cid, num = new[cid], len(area)
    return cid, area


def coarse_pins(pin_cell, pin_off, pin_net, n, cid, num, single):
    """The pins of the cluster problem (src/cluster.py:101-115): each pin's cluster (num: fixed); pins of one-cell
    clusters and fixed pins kept with their offsets, otherwise the first pin of each (net, cluster) at the centre.
    -> (cell, off, net) of the kept pins, in pin order."""
    pin_cell = np.asarray(pin_cell, np.int64)
    owner = np.concatenate([np.asarray(cid, np.int64), [num]])[np.minimum(pin_cell, n)]
    keep_off = np.concatenate([np.asarray(single, bool), [True]])[owner]
    key = np.asarray(pin_net, np.int64) * (num + 1) + owner
    order = np.argsort(key, kind="stable")
    sk = key[order]
    repeat = np.zeros(len(key), bool)
    repeat[order[1:]] = (sk[1:] == sk[:-1]) & ~keep_off[order[1:]]
    sel = ~repeat
    off = np.where(keep_off[sel][:, None], np.asarray(pin_off, np.float32)[sel], np.float32(0))
    return owner[sel], off.astype(np.float32), np.asarray(pin_net, np.int64)[sel]


def expand(cpos, cid, csize, size, draws, num):
    """expand (src/cluster.py:133-144) with the draws [n, 2] given: float32, in the reference's operation order."""
    cpos = np.asarray(cpos, np.float32)
    room = np.maximum(np.asarray(csize, np.float32)[cid] - np.asarray(size, np.float32), np.float32(0))
    cells = cpos[:num][cid] + (np.asarray(draws, np.float32) - np.float32(0.5)) * room
    return np.concatenate([cells, cpos[num:]]).astype(np.float32)


# ------------------------------------------------------------------------------------------------ optimiser
def nesterov_step(u, v, g, lo, hi, alpha, coef):
    """float64: u' = v - alpha g; v' = clamp(u' + coef (u' - u), lo, hi)."""
    u, v, g = (np.asarray(a, np.float64) for a in (u, v, g))
    un = v - float(alpha) * g
    vn = np.minimum(np.maximum(un + float(coef) * (un - u), lo), hi)
    return un, vn


FIELDS = ("lam gam alpha a iter hpwl_prev motion ww mu settled best_hpwl best_ovf is_best improved stop accept "
          "loop_it evals res_hpwl res_ovf has_best").split()
K = {name: i for i, name in enumerate(FIELDS)}
CONSTS = ("base_gamma motion_unit total_pins total_area pitch min_iter stop_ovf settle stall inner refine accuracy "
          "handover").split()
C = {name: i for i, name in enumerate(CONSTS)}
REASON = {1: "converged", 2: "stalled", 3: "diverged", 4: "max_iter", 5: "handover"}


def control(S, kp, c, moved, turned, hpwl, ovf, wa):
    """One pass of the run's control in float64; S [21] and kp [5] updated in place (numpy arrays)."""
    S[K["accept"]] = 0
    S[K["is_best"]] = 0
    if S[K["stop"]] != 0:
        return
    moved, turned, hpwl, ovf, wa = (float(x) for x in (moved, turned, hpwl, ovf, wa))
    if not all(map(math.isfinite, (moved, turned, hpwl, ovf))):
        S[K["stop"]] = 3
        return
    alpha_next = moved / turned if turned > 0 else float(S[K["alpha"]])
    S[K["alpha"]] = alpha_next
    S[K["evals"]] += 1
    S[K["accept"]] = 1
    a = float(S[K["a"]])
    S[K["a"]] = (1 + math.sqrt(4 * a * a + 1)) / 2
    it = float(S[K["iter"]])
    S[K["motion"]] = moved / c[C["motion_unit"]]
    part = float(S[K["lam"]]) * c[C["total_area"]]
    S[K["ww"]] = part / (c[C["total_pins"]] + part)
    if hpwl < S[K["hpwl_prev"]]:
        mu = 1.05 * 0.98
    else:
        mu = 1.05 * max(math.pow(1.05, -float(S[K["motion"]]) * c[C["pitch"]] / float(S[K["gam"]])), 0.95)
    S[K["hpwl_prev"]] = hpwl
    S[K["mu"]] = mu
    S[K["lam"]] *= mu
    if c[C["accuracy"]] != 0:
        err = max(1e-6, 1 - wa / max(hpwl, 1e-12))
        m = max(mu, 1 / mu)
        gn = float(S[K["gam"]]) * min(m, max(1 / m, math.sqrt(max(ovf, 1e-3) / c[C["refine"]] / err)))
        S[K["gam"]] = min(100 * c[C["base_gamma"]], max(0.01 * c[C["base_gamma"]], gn))
    else:
        S[K["gam"]] = c[C["base_gamma"]] * math.pow(10.0, (ovf - 0.1) * 20 / 9 - 1)
    it += 1
    S[K["iter"]] = it
    stop, is_best = 0, 0
    if not (hpwl < 1e30 and ovf < 1e30):
        stop = 3
    else:
        if it >= c[C["min_iter"]] and ovf < c[C["stop_ovf"]]:
            S[K["settled"]] += 1
            is_best = int(hpwl < S[K["best_hpwl"]])
            S[K["best_hpwl"]] = min(hpwl, float(S[K["best_hpwl"]]))
            if S[K["settled"]] > c[C["settle"]]:
                stop = 1
        elif S[K["settled"]] == 0:
            is_best = int(ovf < S[K["best_ovf"]])
            if ovf < S[K["best_ovf"]] * 0.999:
                S[K["improved"]] = it
            S[K["best_ovf"]] = min(ovf, float(S[K["best_ovf"]]))
        if stop == 0:
            if (is_best and S[K["settled"]] > 0) or S[K["ww"]] < 0.95:
                S[K["improved"]] = it
            if it - S[K["improved"]] > c[C["stall"]]:
                stop = 2
        if stop == 0 and c[C["handover"]] > 0 and S[K["lam"]] > 0 and S[K["gam"]] <= c[C["handover"]]:
            stop = 5
    S[K["is_best"]] = is_best
    if is_best:
        S[K["res_hpwl"]] = hpwl
        S[K["res_ovf"]] = ovf
        S[K["has_best"]] = 1
    S[K["loop_it"]] += 1
    if stop == 0 and S[K["loop_it"]] >= c[C["inner"]]:
        stop = 4
    S[K["stop"]] = stop
    if not S[K["has_best"]]:
        S[K["res_hpwl"]] = hpwl
        S[K["res_ovf"]] = ovf
    a = float(S[K["a"]])
    a_next = (1 + math.sqrt(4 * a * a + 1)) / 2
    kp[0] = np.float32(S[K["gam"]])
    kp[1] = np.float32(S[K["lam"]])
    kp[2] = np.float32(S[K["lam"]])
    kp[3] = np.float32(alpha_next)
    kp[4] = np.float32((a - 1) / a_next)


def select(S, u, v, g, u_next, v_next, g_next, best):
    if S[K["accept"]] == 0:
        return
    u[...] = u_next
    v[...] = v_next
    g[...] = g_next
    if S[K["is_best"]] != 0:
        best[...] = v_next


# ------------------------------------------------------------------------------------------------ CPU placement
class CpuLevel(object):
    """One level of global placement on the CPU with the oracle operators (the reference's `--gpu -1` iteration,
    restated): a wirelength-only start, the first density weight in tension units, then the density phase with
    the control rules above. `dtype` is the float type of the wirelength and field arithmetic; `field` = "dct"
    (cosine / sine transforms of the plain map) or "fft" (FFT of the mirrored map, as the reference)."""

    def __init__(self, prob, dtype=np.float64, field="dct", threads=None):
        """threads: run on that many host threads (the *_mt operators: WA in float32, the same map, the same gather;
        transforms by scipy.fft), as the reference's CPU path runs on every core."""
        self.p, self.dtype, self.field = prob, dtype, field
        self.threads = int(threads) if threads else 0
        if self.threads:
            set_threads(self.threads)
        self.evals = 0

    def wirelength(self, pos, gamma):
        cs = self.p.csr
        if self.threads:
            wa, grad, hpwl, _, _ = wa_forward_mt(pos, cs.cell32, cs.off, cs.net_start, cs.cell_start, cs.cell_pin,
                                                 self.p.num_mov, gamma)
            return wa, grad.astype(np.float64), hpwl
        wa, grad, hpwl, _, _ = wa_forward(pos, cs.cell32, cs.off, cs.net_start, self.p.num_mov, gamma, self.dtype)
        return wa, grad, hpwl

    def density(self, pos, wl_grad, weight, precond):
        """-> (gradient [n, 2], overflow on the overflow grid)."""
        p, gr = self.p, self.p.force
        dmap, dgrad = (density_map_mt, density_grad_mt) if self.threads else (density_map, density_grad)
        m = dmap(pos, gr.size, gr.ratio, p.num_mov, gr.bx, gr.by, gr.nbx, gr.nby)
        rho, _, ovsum = density_post(m, gr.fixed_map, gr.target, gr.nbx, gr.nby, mirrored=self.field == "fft")
        overflow = ovsum * gr.bin_area / gr.mov_area
        if p.judge is not None:
            j = p.judge
            mj = dmap(pos[:p.num_mov], j.size, j.ratio, p.num_mov, j.bx, j.by, j.nbx, j.nby)
            _, _, js = density_post(mj, j.fixed_map, j.target, j.nbx, j.nby, mirrored=False)
            overflow = js * j.bin_area / j.mov_area
        if self.field == "fft":
            ex, ey = field_fft(rho, gr.nbx, gr.nby, gr.bin_np, self.dtype, workers=self.threads or None)
        else:
            ex, ey = field_dct(plain_density(m, gr.fixed_map), gr.bin_np)
        g = dgrad(pos, gr.size, gr.ratio, ex, ey, wl_grad, p.pins, p.area, weight, precond, gr.bx, gr.by,
                  gr.nbx, gr.nby)
        return g, overflow

    def grad(self, pos, lam, gam):
        self.evals += 1
        wa, wl, hpwl = self.wirelength(pos, gam)
        if lam == 0:
            g = np.zeros((len(pos), 2))
            g[:self.p.num_mov] = wl / np.maximum(self.p.pins[:self.p.num_mov], 1.0)[:, None]
            return g, wa, hpwl, float("nan")
        g, ovf = self.density(pos, wl, lam, lam)
        return g, wa, hpwl, ovf

    def tension_unit(self, pos):
        g, _ = self.density(pos, None, 1.0, -1.0)
        return float(self.p.pins.astype(np.float64).sum() / np.abs(g[:self.p.num_mov]).sum())

    def run(self, pos0, max_iters=None, time_budget=None, log=None, resume=None, handover_gamma=0.0):
        """Place from pos0 until the stop (or `max_iters` iterations / `time_budget` seconds of the loop).
        resume: dict(lam, gam, iter, hpwl, first_iter): go on where a run on the clusters stopped
        (ParamScheduler.resume, src/param_scheduler.py:53-60): the loop counted from first_iter, no wirelength-only
        start while lam > 0. handover_gamma: stop ("handover") once the smoothing is down to it.
        -> dict(reason, iters, hpwl, overflow, pos, start_iters, seconds, density_iters, iter, lam, gam)."""
        p, o = self.p, self.p.opts
        lo, hi = p.force.pos_lo.astype(np.float64), p.force.pos_hi.astype(np.float64)
        r = resume or {}
        gam, lam = (float(r["gam"]), float(r["lam"])) if resume else (10 * p.base_gamma, 0.0)
        first = int(r.get("first_iter", 0))
        cvec = p.constants(handover_gamma)
        t0 = time.time()
        # estimate_initial_learning_rate + NesterovOptimizer.__init__ (src/nesterov_optimizer.py:15-32,56-61)
        v = np.clip(np.asarray(pos0, np.float64), lo, hi)
        g0 = self.grad(v, lam, gam)[0]
        probe = np.clip(v - o.lr * g0, lo, hi)
        lr = np.linalg.norm(v - probe) / np.linalg.norm(g0 - self.grad(probe, lam, gam)[0])
        g = self.grad(v, lam, gam)[0]
        u = v.copy()
        probe = np.clip(v - lr * g, lo, hi)
        alpha = np.linalg.norm(v - probe) / np.linalg.norm(g - self.grad(probe, lam, gam)[0])
        a = 1.0
        wa_hist, hpwl_hist = [], []
        it_sched, start_iters, reason = int(r.get("iter", 0)), 0, "max_iter"
        it = first
        S = None
        best = None
        hpwl = ovf = float("nan")
        limit = o.inner_iter if max_iters is None else min(o.inner_iter, first + max_iters)
        density_iters = 0
        if lam > 0:                                         # resumed with the density term on
            S = np.zeros(len(FIELDS))
            S[K["lam"]], S[K["gam"]], S[K["alpha"]], S[K["a"]] = lam, gam, alpha, a
            S[K["iter"]], S[K["hpwl_prev"]] = it_sched, float(r["hpwl"])
            S[K["mu"]] = 1.0
            S[K["best_hpwl"]] = S[K["best_ovf"]] = float("inf")
            S[K["loop_it"]] = first
            kp = np.array([gam, lam, lam, alpha, 0.0], np.float32)
            best = v.copy()
        for it in range(first, o.inner_iter):
            if it >= limit or (time_budget is not None and time.time() - t0 > time_budget):
                reason = "sample"
                break
            if S is None:                                   # host phase: the wirelength-only start
                a_next = (1 + math.sqrt(4 * a * a + 1)) / 2
                coef = (a - 1) / a_next
                un, vn = nesterov_step(u, v, g, lo, hi, alpha, coef)
                gn, wa, hpwl, ovf = self.grad(vn, lam, gam)
                moved, turned = np.linalg.norm(vn - v), np.linalg.norm(gn - g)
                if not all(map(math.isfinite, (moved, turned, hpwl))):
                    reason = "diverged"
                    break
                alpha = moved / turned if turned > 0 else alpha
                u, v, g, a = un, vn, gn, a_next
                hpwl_hist.append(hpwl); wa_hist.append(wa); it_sched += 1
                w = 5
                if not (len(wa_hist) <= w or wa_hist[-1 - w] - wa > o.start_tol * w * wa):
                    lam = o.density_weight * self.tension_unit(v)
                    start_iters = it + 1
                    S = np.zeros(len(FIELDS))
                    S[K["lam"]], S[K["gam"]], S[K["alpha"]], S[K["a"]] = lam, gam, alpha, a
                    S[K["iter"]], S[K["hpwl_prev"]] = it_sched, hpwl_hist[-1]
                    S[K["mu"]] = 1.0
                    S[K["best_hpwl"]] = S[K["best_ovf"]] = float("inf")
                    S[K["loop_it"]] = it + 1
                    kp = np.array([gam, lam, lam, alpha, (a - 1) / ((1 + math.sqrt(4 * a * a + 1)) / 2)], np.float32)
                    best = v.copy()
                continue
            density_iters += 1
            un, vn = nesterov_step(u, v, g, lo, hi, kp[3], kp[4])
            gn, wa, hpwl, ovf = self.grad(vn, float(kp[1]), float(kp[0]))
            control(S, kp, cvec, np.linalg.norm(vn - v), np.linalg.norm(gn - g), hpwl, ovf, wa)
            if S[K["accept"]]:
                u, v, g = un, vn, gn
                if S[K["is_best"]]:
                    best = vn.copy()
            if log and int(S[K["loop_it"]]) % log == 0:
                print("iter %d hpwl %.4e ovf %.4f lam %.3e gam %.3e" % (S[K["loop_it"]], hpwl, ovf, S[K["lam"]], S[K["gam"]]))
            if S[K["stop"]]:
                reason = REASON[int(S[K["stop"]])]
                break
        iters = int(S[K["loop_it"]]) if S is not None and reason != "sample" else it
        if S is not None and S[K["has_best"]] and reason != "sample":
            v = best
        res_h = float(S[K["res_hpwl"]]) if S is not None else hpwl
        res_o = float(S[K["res_ovf"]]) if S is not None else ovf
        return dict(reason=reason, iters=iters, hpwl=res_h, overflow=res_o, pos=v, start_iters=start_iters,
                    seconds=time.time() - t0, density_iters=density_iters, evals=self.evals,
                    iter=int(S[K["iter"]]) if S is not None else it_sched,
                    lam=float(S[K["lam"]]) if S is not None else 0.0, gam=float(S[K["gam"]]) if S is not None else gam)


def two_level(prob, pos0, dtype=np.float64, field="dct", threads=None):
    """global_placement_main's two-level branch (src/run_placement.py:87-110) on the CPU: the clusters (cluster_cells
    with the reference's seeded torch draws), their problem (coarse_pins; sizes as squares of the summed area, a
    one-cell cluster keeping its shape; the grid between the overflow grid and the cells' force grid), one level of
    the clusters until the hand-over smoothing (10 x the cells' base gamma), expand, the density weight carried over
    in tension units, then one level of the cells resumed from there.
    -> dict(clusters, coarse_num_bin, coarse_iters, reason, iters, pos, hpwl, overflow)."""
    import torch
    from types import SimpleNamespace
    from autoplace_gb300 import problem as P
    nl, o, n = prob.nl, prob.opts, prob.num_mov
    size = np.asarray(prob.node_size[:n], np.float32)
    area = np.round((size[:, 0] * size[:, 1]).astype(np.float64) * 1024).astype(np.int64)
    gen = torch.Generator().manual_seed(int(o.seed))
    cid, carea = cluster_cells(nl.pin_cell, nl.pin_net, area, o.cluster_ratio,
                               lambda r, num: torch.rand(num, generator=gen).numpy())
    num = len(carea)
    csize = np.repeat(np.sqrt(carea.astype(np.float64) / 1024).astype(np.float32)[:, None], 2, 1)
    single = np.bincount(cid, minlength=num) == 1
    member = np.zeros(num, np.int64)
    member[cid] = np.arange(n)
    csize[single] = size[member[single]]
    c_cell, c_off, c_net = coarse_pins(nl.pin_cell, nl.pin_off, nl.pin_net, n, cid, num, single)
    fine_ff = nl.fixed_fraction(prob.force_bin, prob.force_bin)
    nb = min(prob.force_bin, P.force_num_bin(num, 1.0 - float(fine_ff.mean()), prob.num_bin))
    ff = fine_ff if nb == prob.force_bin else nl.fixed_fraction(nb, nb)
    copts = SimpleNamespace(**vars(o))
    copts.settle_iter, copts.min_iter = 0, 0
    cprob = P.Problem.clusters(prob, csize, c_cell, c_off, c_net, nb, ff, copts)
    pos0 = np.asarray(pos0, np.float32)
    coarse = CpuLevel(cprob, dtype, field, threads)
    level = coarse.run(np.concatenate([pos0[:num], pos0[n:]]), handover_gamma=10 * prob.base_gamma)
    cpos = np.asarray(level["pos"], np.float32)
    gen = torch.Generator().manual_seed(int(o.seed))
    pos = expand(cpos, cid, csize, size, torch.rand(n, 2, generator=gen).numpy(), num)
    pos = np.clip(pos, prob.force.pos_lo, prob.force.pos_hi)
    fine = CpuLevel(prob, dtype, field, threads)
    weight = level["lam"] * fine.tension_unit(pos.astype(np.float64)) / coarse.tension_unit(cpos.astype(np.float64))
    if o.wa_rule == "accuracy":
        gam = level["gam"] / cprob.base_gamma * prob.base_gamma
    else:
        ovf = fine.density(pos.astype(np.float64), None, 1.0, -1.0)[1]
        gam = prob.base_gamma * 10 ** ((ovf - 0.1) * 20 / 9 - 1)
    hpwl = fine.wirelength(pos.astype(np.float64), 10 * prob.base_gamma)[2]
    r = fine.run(pos, resume=dict(lam=weight, gam=gam, iter=level["iter"], hpwl=hpwl, first_iter=level["iters"]))
    return dict(clusters=num, coarse_num_bin=nb, coarse_iters=level["iters"], coarse_reason=level["reason"],
                reason=r["reason"], iters=r["iters"], pos=r["pos"], hpwl=r["hpwl"], overflow=r["overflow"])
