"""How a failure of the tensor-core field reaches the caller, without faulting the GPU.

The field's waits (TMA stages, MMAs, accumulators) are bounded. GP103_OPT_TEST_STALL_FIELD makes the TMA producer
issue no load, so every wait of the field runs out after GP103_OPT_WAIT_MS with nothing in flight. The tests check
that the failure is recorded in the plan's device error flag (gp103_device_error), that the control kernel stops a
pass with reason 6, that the Placer raises RuntimeError, and that the context stays usable: once the flag is cleared,
the same plan gives the correct field again."""
import ctypes

import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


def _plan(nb, mode, bx=7.3, by=6.1):
    """A plan with only the field buffers (gp103_field needs no netlist)."""
    s = native.Sizes()
    native.call("gp103_plan_sizes", nb, nb, mode, ctypes.byref(s))
    keep = dict(c=torch.zeros(s.field_const, dtype=torch.uint8, device=DEV),
                w=torch.zeros(s.field_work, dtype=torch.uint8, device=DEV),
                red=torch.zeros(s.red, dtype=torch.float64, device=DEV),
                cnt=torch.zeros(16, dtype=torch.int32, device=DEV),
                map=torch.zeros((2, nb, nb), dtype=torch.int64, device=DEV),
                ex=torch.zeros((nb, nb), device=DEV), ey=torch.zeros((nb, nb), device=DEV),
                kp=torch.zeros(5, device=DEV))
    pl = native.Plan()
    pl.nbx = pl.nby = nb
    pl.bx, pl.by = bx, by
    pl.field_mode = mode
    pl.field_const, pl.field_work = keep["c"].data_ptr(), keep["w"].data_ptr()
    pl.red, pl.counters, pl.map = keep["red"].data_ptr(), keep["cnt"].data_ptr(), keep["map"].data_ptr()
    pl.ex, pl.ey, pl.kp = keep["ex"].data_ptr(), keep["ey"].data_ptr(), keep["kp"].data_ptr()
    native.call("gp103_field_constants", ctypes.byref(pl), torch.cuda.current_stream().cuda_stream)
    return pl, keep


class _Stalled(object):
    """The field's waits run out after `ms` milliseconds (the options are process-wide: restored on exit)."""

    def __init__(self, ms=5):
        self.ms = ms

    def __enter__(self):
        native.call("gp103_set_option", native.OPT_WAIT_MS, self.ms)
        native.call("gp103_set_option", native.OPT_TEST_STALL_FIELD, 1)

    def __exit__(self, *exc):
        native.call("gp103_set_option", native.OPT_TEST_STALL_FIELD, 0)
        native.call("gp103_set_option", native.OPT_WAIT_MS, 2000)


def test_wait_options_are_checked():
    lib = native.lib()
    assert lib.gp103_set_option(native.OPT_WAIT_MS, 0) == native.ERR_ARG
    assert lib.gp103_set_option(native.OPT_WAIT_MS, 60001) == native.ERR_ARG
    assert lib.gp103_set_option(99, 1) == native.ERR_ARG


@pytest.mark.parametrize("nb", [256, 384])
def test_field_timeout_is_reported_and_cleared(nb):
    """256: the folded f16x3 transforms; 384: the unfolded ones."""
    s = torch.cuda.current_stream().cuda_stream
    pl, keep = _plan(nb, native.FIELD_F16X3)
    rng = np.random.default_rng(3)
    a = rng.random((nb, nb)) * 0.3 + 0.6
    a[nb // 3: nb // 3 + 5, nb // 2: nb // 2 + 7] += 40.0                   # a clump
    a = a.astype(np.float32)
    d = torch.as_tensor(a).to(DEV)
    ex, ey = torch.full((nb, nb), 7.0, device=DEV), torch.full((nb, nb), 7.0, device=DEV)
    assert native.device_error(ctypes.byref(pl), s) == 0
    with _Stalled():
        native.call("gp103_field", ctypes.byref(pl), d.data_ptr(), ex.data_ptr(), ey.data_ptr(), s)
        code = native.device_error(ctypes.byref(pl), s)
    assert code in native.DEVICE_ERRORS, code
    # the flag stays set until cleared: a later launch gives up at once and stores nothing
    native.call("gp103_field", ctypes.byref(pl), d.data_ptr(), ex.data_ptr(), ey.data_ptr(), s)
    assert native.device_error(ctypes.byref(pl), s) == code
    assert bool((ex == 7.0).all()) and bool((ey == 7.0).all())        # the last GEMM stored nothing
    assert native.device_error(ctypes.byref(pl), s, clear=True) == code
    assert native.device_error(ctypes.byref(pl), s) == 0
    # the context and the plan are usable again
    native.call("gp103_field", ctypes.byref(pl), d.data_ptr(), ex.data_ptr(), ey.data_ptr(), s)
    torch.cuda.synchronize()
    assert native.device_error(ctypes.byref(pl), s) == 0
    fx, fy = O.field_dct(a, np.array([7.3, 6.1]))
    scale = max(np.abs(fx).max(), np.abs(fy).max())
    err = max(np.abs(ex.cpu().numpy() - fx).max(), np.abs(ey.cpu().numpy() - fy).max()) / scale
    assert err <= 1e-6, err


def _small_problem():
    nl = synth.make_netlist(3000, 3150, window=80, macros=3, cover=0.1, fixed_pin_share=0.02, seed=5)
    return problem.Problem(nl, problem.options(target_density=0.9, num_bin=64, force_num_bin=128)), nl


def test_pass_stops_with_device_error_and_placer_raises():
    from autoplace_gb300.engine import Placer, SK, STOP_DEVICE_ERROR
    prob, nl = _small_problem()
    pl = Placer(prob, field="f16x3", use_graphs=False)
    assert pl.mode == native.FIELD_F16X3
    with torch.cuda.stream(pl.stream):
        pl.V[0].copy_(torch.as_tensor(synth.init_positions(nl, prob.num_nodes, seed=5)).to(DEV))
    # a density pass whose field gives up: the control stops the run (reason 6) and accepts nothing
    with _Stalled():
        pl._passes(native.PHASE_DENSITY, 1)
    pl.sync()
    S = pl.S.cpu().numpy()
    assert S[SK["stop"]] == STOP_DEVICE_ERROR and S[SK["accept"]] == 0
    # the start phase's control stops too while the flag is set
    pl._passes(native.PHASE_START, 1)
    pl.sync()
    assert pl.T.cpu().numpy()[native.T["stop"]] == STOP_DEVICE_ERROR
    with pytest.raises(RuntimeError, match="device error"):
        pl.check_device()
    # an evaluation with the density term raises while the flag is set
    out = torch.zeros_like(pl.V[0])
    with pytest.raises(RuntimeError, match="tensor-core field"):
        pl.eval(pl.V[0], out, weight=1e-3, precond=1e-3)
    assert pl.clear_device_error() != 0
    # cleared: the same Placer places normally
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=5)
    r = pl.run(torch.as_tensor(pos0).to(DEV))
    assert r["reason"] in ("converged", "stalled")
    assert pl.clear_device_error() == 0


def test_run_raises_when_the_field_fails():
    """A whole run with the field stalled from the start: RuntimeError, not a placement on stale fields."""
    from autoplace_gb300.engine import Placer
    prob, nl = _small_problem()
    pos0 = torch.as_tensor(synth.init_positions(nl, prob.num_nodes, seed=5)).to(DEV)
    with _Stalled():
        pl = Placer(prob, field="f16x3")
        with pytest.raises(RuntimeError, match="device error"):
            pl.run(pos0)
