"""Autotuner: the per-instance choices of the fused pass, picked by timing them on the GPU.

The reference has one launch rule for every kernel (a block of 256 threads per item, cpp_to_py/gp_cuda_kernel.cu:5-6).
Here two choices depend on the instance and are measured, not guessed:
  - the field mode of the force grid: the tensor-core f16x3 GEMMs (grids of multiples of 128 bins) or the float32
    CUDA-core GEMMs (any grid; on small grids the tensor-core form's fixed costs can dominate);
  - the WA kernels' lane groups, i.e. the degree thresholds between one thread per net, groups of 4 / 8 / 16 lanes and
    a warp per net. The nets are ordered by degree class at set-up, so every partition of the class boundaries below
    is a valid launch: "default" (<= 8 pins a thread, 9-16 four lanes, longer a warp), "groups" (as default, and 17-32
    pins eight lanes, 33-64 sixteen), "warp" (every net of more than 8 pins a warp), "wide" (9-32 pins eight lanes,
    33-64 sixteen).
Each candidate runs `passes` density passes (after `warm` untimed ones) from a mid-run state of the instance; the
fastest per-pass time wins. Results are cached by the instance's size class (cells rounded to a power of 2, grid).
"""
import math

import torch

from . import native
from .engine import Placer

WA_CHOICES = ("default", "groups", "warp", "wide")
_CACHE = {}


def apply_wa(placer, choice):
    """Set the WA class boundaries of a Placer's plan (from the ones its net order found)."""
    pl = placer.plan
    if not hasattr(placer, "_wa_bounds"):
        placer._wa_bounds = (pl.net_split, pl.net_mid, placer.net_g8, placer.net_g16)
    split, mid, g8, g16 = placer._wa_bounds
    if choice == "default":
        pl.net_mid, pl.net_g8, pl.net_g16 = mid, 0, 0
    elif choice == "groups":
        pl.net_mid, pl.net_g8, pl.net_g16 = mid, g8, g16
    elif choice == "warp":
        pl.net_mid, pl.net_g8, pl.net_g16 = split, split, 0
    elif choice == "wide":
        pl.net_mid, pl.net_g8, pl.net_g16 = split, g8, g16
    else:
        raise ValueError(choice)
    if pl.net_g16 == 0:
        pl.net_g8 = 0
    placer._graphs = {}                                  # captured passes hold the old boundaries


def _time_passes(placer, passes, warm):
    s = placer.stream
    placer._passes(native.PHASE_DENSITY, warm)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    placer._passes(native.PHASE_DENSITY, passes)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / passes


def _state(placer, pos0):
    """A mid-run state: the wirelength-only start, the first density weight, 48 density passes."""
    ctx = placer.begin(pos0)
    if ctx["start"]:
        for _ in range(100):
            placer._passes(native.PHASE_START, 4)
            placer.sync()
            T = placer.T.cpu().numpy()
            if T[native.T["done"]] or T[native.T["stop"]]:
                break
        placer.start_end(ctx)
    placer._passes(native.PHASE_DENSITY, 48)
    placer.sync()


def key(prob):
    return (int(round(math.log2(max(prob.num_mov, 1)))), prob.force.nbx, prob.force.nby)


def tune(prob, pos0, fields=("f16x3", "fp32"), passes=16, warm=4, device="cuda", log=None):
    """-> dict(field, wa, ms_per_pass, table) for the instance (cached by size class)."""
    k = key(prob)
    if k in _CACHE:
        return _CACHE[k]
    table = {}
    best = None
    for f in fields:
        pl = Placer(prob, field=f, device=device, use_graphs=False)
        if native.FIELD_MODES[f] != pl.mode:             # the grid does not take this mode
            continue
        _state(pl, pos0)
        for w in WA_CHOICES:
            apply_wa(pl, w)
            ms = _time_passes(pl, passes, warm)
            table["%s/%s" % (f, w)] = ms
            if best is None or ms < best[2]:
                best = (f, w, ms)
        del pl
    out = dict(field=best[0], wa=best[1], ms_per_pass=best[2], table=table)
    if log:
        log("tuned %s: %s" % (k, out))
    _CACHE[k] = out
    return out
