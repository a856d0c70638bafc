"""Host-side checks that need no GPU: the C-ABI library loads and exports what include/gp103.h declares, the
ctypes plan matches the C struct, and the host logic of the engine (net reordering) is exact."""
import ctypes
import os
import re

import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from autoplace_gb300.engine import G8_NET, G16_NET, MID_NET, SHORT_NET, net_order

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "gp103.h")).read()
    return sorted(set(re.findall(r"\b(gp103_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = native.lib()
    declared = header_functions()
    assert declared, "no function declared"
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(native.exported_symbols())
    assert L.gp103_version() >= 1
    assert L.gp103_status_string(1).decode().startswith("invalid argument")


def test_plan_layout_matches_c_struct():
    n = len(native.Plan._fields_)
    out = (ctypes.c_size_t * (n + 1))()
    count = native.lib().gp103_plan_offsets(out, n + 1)
    assert count == n
    for k, (name, _) in enumerate(native.Plan._fields_):
        assert getattr(native.Plan, name).offset == out[k], name
    assert ctypes.sizeof(native.Plan) == out[n]


def test_plan_sizes_and_shape_errors():
    s = native.Sizes()
    native.call("gp103_plan_sizes", 256, 256, native.FIELD_BF16X6, ctypes.byref(s))
    assert s.field_const > 6 * 256 * 256 * 6 and s.field_work > 0 and s.red > 0
    assert native.lib().gp103_plan_sizes(96, 96, native.FIELD_BF16X6, ctypes.byref(s)) == native.ERR_SHAPE
    native.call("gp103_plan_sizes", 96, 96, native.FIELD_FP32, ctypes.byref(s))
    with pytest.raises(RuntimeError, match="invalid argument"):
        native.call("gp103_plan_sizes", 0, 96, native.FIELD_FP32, ctypes.byref(s))
    # tf32x3: two float32 term planes per operand (8 bytes an element), on the tensor cores' grids only
    native.call("gp103_plan_sizes", 256, 256, native.FIELD_TF32X3, ctypes.byref(s))
    assert s.field_const > 6 * 256 * 256 * 8 and s.field_work > 6 * 256 * 256 * 8
    assert native.lib().gp103_plan_sizes(96, 96, native.FIELD_TF32X3, ctypes.byref(s)) == native.ERR_SHAPE
    with pytest.raises(RuntimeError, match="invalid argument"):
        native.call("gp103_plan_sizes", 256, 256, 5, ctypes.byref(s))


def test_device_limits_equal_host_limits():
    """The clustering's merge limits from the areas as the device computes them (integer sums, then the reference's
    float32 scalar arithmetic) equal the host statement's, here on CPU tensors."""
    import numpy as np
    import torch
    from autoplace_gb300 import cluster
    rng = np.random.default_rng(3)
    for n, hi in ((10, 50), (100_000, 9 * 1024 * 10), (7, 3)):
        area = rng.integers(1, hi, n).astype(np.int64)
        area[: n // 50] *= 40                   # a few cells at or above the lone-cell bound
        for ratio in (5.0, 3.0, 1.5):
            assert cluster.device_limits(torch.as_tensor(area), ratio) == cluster.limits(area, ratio)


def test_handover_bound_never_overshoots():
    """The lower bound on the passes before the clusters' hand-over (Placer._handover_bound) is at most the passes
    the fastest smoothing decrease the accuracy rule allows (a factor 1 / 1.05 per pass, in float64) takes."""
    from types import SimpleNamespace
    from autoplace_gb300 import engine
    SK = engine.SK
    fake = SimpleNamespace(handover_gamma=2.0, p=SimpleNamespace(opts=SimpleNamespace(wa_rule="accuracy")))
    for g0 in (2.0, 2.05, 2.1, 3.0, 17.0, 400.0, 1e4):
        Sh = [0.0] * len(engine.S_FIELDS)
        Sh[SK["lam"]], Sh[SK["gam"]] = 1e-3, g0
        bound = engine.Placer._handover_bound(fake, Sh)
        g, passes = g0, 0
        while g > fake.handover_gamma:
            g = g * (1.0 / 1.05)
            passes += 1
        assert 1 <= bound <= max(passes, 1), (g0, bound, passes)
    Sh = [0.0] * len(engine.S_FIELDS)
    Sh[SK["gam"]] = 10.0                        # no density weight yet: no hand-over bound
    assert engine.Placer._handover_bound(fake, Sh) is None
    fake.p.opts.wa_rule = "overflow"            # the overflow rule's smoothing is not bounded per pass
    Sh[SK["lam"]] = 1e-3
    assert engine.Placer._handover_bound(fake, Sh) is None


def test_wa_long_share_rule():
    """The fused WA launch's long-net share from the share of the pins on long nets: 30 + 60 f within 40 .. 75."""
    from autoplace_gb300 import engine
    assert engine.wa_long_share(0, 0) == 0
    assert engine.wa_long_share(1000, 620) == 53          # 38 % of the pins on long nets (the 1.2M-cell netlist)
    assert engine.wa_long_share(1000, 470) == 62          # 53 % (its clusters)
    assert engine.wa_long_share(1000, 1000) == 40 and engine.wa_long_share(1000, 0) == 75


def test_argument_errors_without_gpu():
    """Bad sizes are rejected before any launch (no GPU needed)."""
    L = native.lib()
    assert L.gp103_wa(None, None, None, None, None, None, -1, 0, None, None, None, None, None) == native.ERR_ARG
    assert L.gp103_density_map(None, None, None, 0, 0, 1.0, 1.0, 0, 4, None, None, 1.0, None, None,
                               None) == native.ERR_ARG
    assert L.gp103_select(None, None, None, None, None, None, None, None, 0, None) == native.ERR_ARG
    assert L.gp103_hpwl(None, None, None, None, 5, 3, None, None, None) == native.ERR_ARG
    assert L.gp103_exact_overflow(None, None, 3, 1.0, 1.0, 0, 8, None, 1.0, 1.0, None, None, None,
                                  None) == native.ERR_ARG


def test_net_order_keeps_nets_and_cell_sums():
    nl = synth.make_netlist(3000, 3100, window=60, macros=3, cover=0.1, fixed_pin_share=0.05, seed=4)
    cs = problem.build_csr(nl.pin_cell, nl.pin_off, nl.pin_net, nl.num_nets, nl.num_mov, 100)
    perm, ns, slot, split, mid, two, three, g8, g16 = net_order(cs.net_start, cs.cell32, cs.cell_pin)
    deg = np.diff(ns)
    assert np.all(deg[:split] <= SHORT_NET) and np.all(deg[split:] > SHORT_NET)
    assert np.all(deg[split:mid] <= MID_NET) and np.all(deg[mid:] > MID_NET)
    assert np.all(deg[mid:g8] <= G8_NET) and np.all(deg[g8:] > G8_NET)
    assert np.all(deg[g8:g16] <= G16_NET) and np.all(deg[g16:] > G16_NET)
    assert np.all(deg[:two] == 2) and np.all(deg[two:three] == 3) and np.all(deg[three:] > 3)
    assert two > 0 and three > two and g16 > g8 > mid
    cls = np.select([deg == 2, deg == 3, deg <= SHORT_NET, deg <= MID_NET, deg <= G8_NET, deg <= G16_NET],
                    [0, 1, 2, 3, 4, 5], 6)
    assert np.all(np.diff(cls) >= 0)                       # classes in order
    assert sorted(perm.tolist()) == list(range(len(perm)))  # a permutation of the pins
    assert sorted(slot.tolist()) == list(range(len(slot)))
    # every net keeps its pins, in order: the new nets are the old ones, each once
    old_of_new = perm[ns[:-1]]
    starts = set(cs.net_start[:-1].tolist())
    assert set(old_of_new.tolist()) == starts
    for k in range(0, len(deg), 97):
        i = int(np.searchsorted(cs.net_start, perm[ns[k]]))
        assert np.array_equal(perm[ns[k]:ns[k + 1]], np.arange(cs.net_start[i], cs.net_start[i + 1]))
    # the pin at new position q sits at slot[q] in cell order, which lists the old pins as cell_pin does
    cell_order = np.empty(len(perm), np.int64)
    cell_order[slot] = perm
    assert np.array_equal(cell_order, cs.cell_pin)
    # short nets of one class are ordered by their lowest cell
    first = np.minimum.reduceat(cs.cell32[perm], ns[:-1])
    for c in range(7):
        f = first[cls == c]
        assert np.all(np.diff(f) >= 0)


def test_field_mode_falls_back_to_fp32_on_small_grids():
    """A tensor-core field needs multiples of 128 bins per side: smaller grids (clusters, small designs) run the
    fp32 field (decided by gp103_plan_sizes, host only)."""
    from autoplace_gb300.engine import field_mode
    assert field_mode(native.FIELD_BF16X6, 32, 32) == native.FIELD_FP32
    assert field_mode(native.FIELD_BF16X3, 64, 128) == native.FIELD_FP32
    assert field_mode(native.FIELD_BF16X6, 256, 128) == native.FIELD_BF16X6
    assert field_mode(native.FIELD_FP32, 256, 256) == native.FIELD_FP32
