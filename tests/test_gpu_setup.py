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
    split = torch.zeros(2, dtype=torch.int32, device=DEV)
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
    perm, new_start, slot, split, mid = net_order(cs.net_start, cs.cell32, cs.cell_pin)
    ns_d, cell_d, off_d, slot_d, split_d = device_order(cs, nl.num_mov)
    assert np.array_equal(ns_d, new_start)
    assert np.array_equal(cell_d, cs.cell32[perm])
    assert np.array_equal(off_d.view(np.uint32), cs.off[perm].view(np.uint32))
    assert np.array_equal(slot_d, slot)
    assert split_d == [split, mid]


def test_device_net_order_empty():
    cs = problem.build_csr(np.zeros(0, np.int64), np.zeros((0, 2), np.float32), np.zeros(0, np.int64), 0, 10, 100)
    ns_d, _, _, _, split_d = device_order(cs, 10)
    assert ns_d.tolist() == [0] and split_d == [0, 0]
