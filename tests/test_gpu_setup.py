"""The device net order (gp103_net_order) against the host restatement engine.net_order: the same permutation of
nets and pins, the same slots, the same split (integer work: bit-exact)."""
import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from autoplace_gb300.engine import net_order

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a)).to(DEV)


def device_order(cs, num_mov):
    P, N = len(cs.cell32), cs.num_nets
    ns_out = torch.zeros(N + 1, dtype=torch.int32, device=DEV)
    cell_out = torch.zeros(max(P, 1), dtype=torch.int32, device=DEV)
    off_out = torch.zeros((max(P, 1), 2), dtype=torch.float32, device=DEV)
    slot = torch.zeros(max(P, 1), dtype=torch.int32, device=DEV)
    split = torch.zeros(6, dtype=torch.int32, device=DEV)
    nbytes = int(native.lib().gp103_net_order_scratch(N, P, num_mov))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=DEV)
    ins = [cu(cs.net_start), cu(cs.cell32), cu(cs.off), cu(cs.cell_pin)]
    native.call("gp103_net_order", *(x.data_ptr() for x in ins), N, P, num_mov, scratch.data_ptr(), nbytes,
                ns_out.data_ptr(), cell_out.data_ptr(), off_out.data_ptr(), slot.data_ptr(), split.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return (ns_out.cpu().numpy(), cell_out.cpu().numpy()[:P], off_out.cpu().numpy()[:P], slot.cpu().numpy()[:P],
            split.cpu().tolist())


@pytest.mark.parametrize("cells,seed", [(3000, 0), (20000, 7)])
def test_device_net_order_matches_host(cells, seed):
    nl = synth.make_netlist(cells, int(cells * 1.05), window=200, macros=2, cover=0.1, seed=seed)
    cs = problem.build_csr(nl.pin_cell, nl.pin_off, nl.pin_net, nl.num_nets, nl.num_mov, 100)
    perm, new_start, slot, *bounds = net_order(cs.net_start, cs.cell32, cs.cell_pin)
    split, mid, two, three, g8, g16 = bounds
    ns_d, cell_d, off_d, slot_d, split_d = device_order(cs, nl.num_mov)
    assert np.array_equal(ns_d, new_start)
    assert np.array_equal(cell_d, cs.cell32[perm])
    assert np.array_equal(off_d.view(np.uint32), cs.off[perm].view(np.uint32))
    assert np.array_equal(slot_d, slot)
    assert split_d == list(bounds)
    deg = np.diff(new_start)
    assert (deg[:two] == 2).all() and (deg[two:three] == 3).all() and (deg[three:] > 3).all()


def test_device_net_order_empty():
    cs = problem.build_csr(np.zeros(0, np.int64), np.zeros((0, 2), np.float32), np.zeros(0, np.int64), 0, 10, 100)
    ns_d, _, _, _, split_d = device_order(cs, 10)
    assert ns_d.tolist() == [0] and split_d == [0] * 6


def _same(a, b):
    a = a.cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape and a.dtype.itemsize == b.dtype.itemsize
    return np.array_equal(a.view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def _check_device_problem(nl, opts):
    hp = problem.Problem(nl, opts)
    dp = problem.Problem(nl, opts, arrays=False).on_device()
    hc, dc = hp.csr, dp.csr
    assert dc.num_nets == hc.num_nets
    for k in ("net_start", "cell32", "off", "cell_start", "cell_pin"):
        assert _same(getattr(dc, k), getattr(hc, k)), k
    for k in ("all_cell", "all_off", "all_net_start", "pins", "area"):
        assert _same(getattr(dp, k), getattr(hp, k)), k
    for g in ("force", "judge"):
        if getattr(hp, g) is None:
            assert getattr(dp, g) is None
            continue
        for k in ("size", "ratio", "pos_lo", "pos_hi"):
            assert _same(getattr(getattr(dp, g), k), getattr(getattr(hp, g), k)), (g, k)
    assert dp.total_pins == hp.total_pins
    assert np.array_equal(dp.constants(), hp.constants())
    return hp, dp


@pytest.mark.parametrize("cells,seed,ignore", [(3000, 0, 100), (20000, 7, 100), (20000, 3, 6)])
def test_device_problem_build_matches_host(cells, seed, ignore):
    """The net filter, CSR, cell order, every net's start and the smoothed nodes built on the device
    (gp103_build_csr, gp103_smooth_nodes) against the host build: bit for bit."""
    nl = synth.make_netlist(cells, int(cells * 1.05), window=200, macros=3, cover=0.1, fixed_pin_share=0.02,
                            seed=seed)
    _check_device_problem(nl, problem.options(target_density=0.9, num_bin=64, force_num_bin=128,
                                              ignore_net_degree=ignore))


def test_device_problem_build_big_cells_and_placement():
    """Cells of many pins (33 .. a few thousand: the block-sorted path) keep their pins in pin order; the Placer runs
    the device-built problem to the same placement as the host-built one."""
    from autoplace_gb300.engine import Placer
    nl = synth.make_netlist(6000, 6300, window=150, macros=2, cover=0.1, fixed_pin_share=0.02, seed=5)
    pc = np.array(nl.pin_cell)
    movable = np.flatnonzero(pc < nl.num_mov)
    pc[movable[::40]] = 7                           # one cell with ~500 pins
    pc[movable[5::97]] = 11                         # another with ~200
    pc[movable[3:200:5]] = 13                       # and one with 40
    nl.pin_cell = pc
    hp, dp = _check_device_problem(nl, problem.options(target_density=0.9, num_bin=64, force_num_bin=128))
    assert np.diff(hp.csr.cell_start)[[7, 11, 13]].min() > 32
    pos0 = synth.init_positions(nl, hp.num_nodes, seed=1)
    rh = Placer(hp, field="fp32").run(pos0)
    rd = Placer(dp, field="fp32").run(pos0)
    assert rh["iters"] == rd["iters"] and rh["reason"] == rd["reason"]
    assert np.array_equal(rh["pos"].cpu().numpy(), rd["pos"].cpu().numpy())


def test_device_problem_build_rejects_bad_pins():
    """An unsorted pin_net or a pin on a cell out of range: the device build raises (the kernels stay in bounds)."""
    nl = synth.make_netlist(2000, 2100, window=100, macros=0, seed=2)
    opts = problem.options(target_density=1.0, num_bin=32)
    base = problem.Problem(nl, opts, arrays=False)
    src = problem.netlist_arrays(base)
    bad = dict(src, pin_net=src["pin_net"].copy())
    bad["pin_net"][[10, 400]] = bad["pin_net"][[400, 10]]
    with pytest.raises(ValueError, match="not sorted"):
        base.on_device(host=bad)
    bad = dict(src, pin_cell=src["pin_cell"].copy())
    bad["pin_cell"][17] = nl.num_mov + 5
    with pytest.raises(ValueError, match="cell out of range"):
        base.on_device(host=bad)


@pytest.mark.parametrize("ignore", [1, 2, 3])
def test_device_problem_build_filters(ignore):
    """Degree filters that keep no net (1), only the 2-pin nets (2) or the 2- and 3-pin nets (3): the device build
    equals the host build, empty CSR included."""
    nl = synth.make_netlist(2000, 2100, window=100, macros=2, cover=0.1, fixed_pin_share=0.05, seed=8)
    hp, dp = _check_device_problem(nl, problem.options(target_density=0.9, num_bin=64, force_num_bin=128,
                                                       ignore_net_degree=ignore))
    if ignore == 1:
        assert dp.csr.num_nets == 0 and len(dp.csr.cell32) == 0


@pytest.mark.parametrize("nb", [(64, 64), (512, 256), (1024, 1024)])
def test_device_fixed_fraction_is_bit_exact(nb):
    """The fixed share of the bins on the device (gp103_macro_fraction) against the host statement, bit for bit; with
    and without macros, on square and non-square grids."""
    from autoplace_gb300.cluster import device_fixed_fraction
    for macros, cover in ((40, 0.2), (0, 0.0), (3, 0.12)):
        nl = synth.make_netlist(20000, 21000, window=200, macros=macros, cover=cover, seed=macros + 1)
        host = nl.fixed_fraction(*nb)
        dev = device_fixed_fraction(nl, *nb)
        assert dev.shape == host.shape and np.array_equal(dev.view(np.uint64), host.view(np.uint64))
