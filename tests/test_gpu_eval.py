"""The exact evaluators (float64 HPWL over every net, overflow of the real-size cells) against the oracle."""
import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth
from oracle import gp_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a)).to(DEV)


def _case(seed, cells=4000, nb=64):
    nl = synth.make_netlist(cells, cells + 200, window=80, macros=3, cover=0.12, seed=seed)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=nb // 2, force_num_bin=nb))
    rng = np.random.default_rng(seed)
    pos = (rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]).astype(np.float32)
    pos[:cells // 4] = pos[:cells // 4] * 0.02 + np.array([nl.width * 0.3, nl.height * 0.6], np.float32)
    return nl, prob, pos


def _hpwl(prob, pos, num_nets=None):
    scratch = torch.zeros(native.EVAL_SCRATCH_BYTES, dtype=torch.uint8, device=DEV)
    out = torch.zeros(1, dtype=torch.float64, device=DEV)
    ns = prob.all_net_start if num_nets is None else prob.all_net_start[:num_nets + 1]
    p, c, o, s = cu(pos), cu(prob.all_cell), cu(prob.all_off), cu(ns)
    native.call("gp103_hpwl", p.data_ptr(), c.data_ptr(), o.data_ptr(), s.data_ptr(), len(ns) - 1, prob.num_mov,
                scratch.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return float(out.item())


@pytest.mark.parametrize("seed", [0, 3])
def test_exact_hpwl_matches_oracle(seed):
    nl, prob, pos = _case(seed)
    ref = O.hpwl_all(pos, prob.all_cell, prob.all_off, prob.all_net_start, prob.num_mov)
    got = _hpwl(prob, pos)
    assert abs(got - ref) <= 1e-12 * abs(ref)
    assert _hpwl(prob, pos, num_nets=0) == 0.0


@pytest.mark.parametrize("seed", [1, 4])
def test_exact_overflow_matches_oracle(seed):
    nl, prob, pos = _case(seed)
    gr = prob.real_judge
    C = prob.num_mov
    size = np.ascontiguousarray(nl.size, dtype=np.float32)
    scale = gr.bin_area / gr.mov_area
    om = O.density_map(pos[:C], size, np.ones(C, np.float32), C, gr.bx, gr.by, gr.nbx, gr.nby)
    _, _, total = O.density_post(om, gr.fixed_map, gr.target, gr.nbx, gr.nby, mirrored=False)
    ref = total * scale
    m = torch.zeros((gr.nbx, gr.nby), dtype=torch.int64, device=DEV)
    scratch = torch.zeros(native.EVAL_SCRATCH_BYTES, dtype=torch.uint8, device=DEV)
    out = torch.zeros(1, dtype=torch.float64, device=DEV)
    p, s, f = cu(pos), cu(size), cu(gr.fixed_map)
    for _ in range(2):          # the map is left zeroed: a second call gives the same value
        native.call("gp103_exact_overflow", p.data_ptr(), s.data_ptr(), C, gr.bx, gr.by, gr.nbx, gr.nby,
                    f.data_ptr(), gr.target, scale, m.data_ptr(), scratch.data_ptr(), out.data_ptr(),
                    torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert abs(float(out.item()) - ref) <= 1e-12 * max(abs(ref), 1e-30)
        assert int(m.abs().sum().item()) == 0
