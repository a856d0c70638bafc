"""gp103_density_map_noalloc, the density map for callers that cannot allocate device memory (a plugin inside a host
application whose device memory belongs to that application's pool, a loop that must not call cudaMalloc because it
can synchronise the device). Its scratch is a fixed array inside the library; its results must be those of
gp103_density_map, which takes a caller-provided scratch map. Collected last (file name), so that a failure here
leaves every other test already run; it also passes on its own in a fresh process."""
import numpy as np
import pytest

from autoplace_gb300 import native, problem, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case(seed, cells, nb):
    nl = synth.make_netlist(cells, cells + 50, window=60, macros=2, cover=0.1, seed=seed)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=nb, force_num_bin=nb))
    gr = prob.force
    rng = np.random.default_rng(seed)
    pos = rng.random((prob.num_nodes, 2)) * [nl.width, nl.height]
    pos[: cells // 4] = pos[: cells // 4] * 0.02 + [nl.width * 0.4, nl.height * 0.5]      # a clump
    pos = np.clip(pos, gr.pos_lo, gr.pos_hi).astype(np.float32)
    return prob, gr, pos


def _inputs(prob, gr, pos):
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()
    return t(pos), t(gr.size), t(gr.ratio), t(gr.fixed_map)


def _with_scratch(prob, gr, args):
    p, s, r, f = args
    m = torch.empty((2, gr.nbx, gr.nby), dtype=torch.int64, device="cuda")
    rho = torch.empty((2 * gr.nbx, 2 * gr.nby), device="cuda")
    over = torch.empty((gr.nbx, gr.nby), device="cuda")
    native.call("gp103_density_map", p.data_ptr(), s.data_ptr(), r.data_ptr(), p.shape[0], prob.num_mov, gr.bx, gr.by,
                gr.nbx, gr.nby, m.data_ptr(), f.data_ptr(), gr.target, rho.data_ptr(), over.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    return rho, over


def _no_alloc(prob, gr, args):
    p, s, r, f = args
    rho = torch.empty((2 * gr.nbx, 2 * gr.nby), device="cuda")
    over = torch.empty((gr.nbx, gr.nby), device="cuda")
    native.call("gp103_density_map_noalloc", p.data_ptr(), s.data_ptr(), r.data_ptr(), p.shape[0], prob.num_mov,
                gr.bx, gr.by, gr.nbx, gr.nby, f.data_ptr(), gr.target, rho.data_ptr(), over.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    return rho, over


def test_no_alloc_density_map_matches_the_scratch_version():
    """Two calls in a row (different grids and nodes; the second must not see the first one's sums) give what
    gp103_density_map gives: the same integer map, so bit-identical density and overflow maps (tolerance 0)."""
    for seed, cells, nb in ((3, 4000, 128), (4, 9000, 256)):
        prob, gr, pos = _case(seed, cells, nb)
        args = _inputs(prob, gr, pos)
        want_rho, want_over = _with_scratch(prob, gr, args)
        got_rho, got_over = _no_alloc(prob, gr, args)
        torch.cuda.synchronize()
        assert torch.equal(got_rho, want_rho)
        assert torch.equal(got_over, want_over)


def test_no_alloc_rejects_grids_beyond_its_scratch():
    prob, gr, pos = _case(5, 500, 16)
    p, s, r, f = _inputs(prob, gr, pos)
    big = 1024                                                   # 1024 x 1024 > 262,144 bins
    rho = torch.empty(1, device="cuda")
    st = native.lib().gp103_density_map_noalloc(p.data_ptr(), s.data_ptr(), r.data_ptr(), p.shape[0], prob.num_mov,
                                                gr.bx, gr.by, big, big, f.data_ptr(), gr.target, rho.data_ptr(),
                                                rho.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 4
    assert "262144" in native.lib().gp103_status_string(st).decode()


def test_no_alloc_at_the_limit_and_with_no_nodes():
    """A grid of exactly 262,144 bins (512 x 512, the array's size) is bit-identical to gp103_density_map; then a call
    with no nodes after it gives the fixed map alone (the array's leftover sums are cleared)."""
    prob, gr, pos = _case(6, 30000, 512)
    assert gr.nbx * gr.nby == 262144
    args = _inputs(prob, gr, pos)
    want_rho, want_over = _with_scratch(prob, gr, args)
    got_rho, got_over = _no_alloc(prob, gr, args)
    torch.cuda.synchronize()
    assert torch.equal(got_rho, want_rho) and torch.equal(got_over, want_over)
    p, s, r, f = args
    empty = (p[:0], s[:0], r[:0], f)
    want_rho, want_over = _with_scratch(prob, gr, empty)
    got_rho, got_over = _no_alloc(prob, gr, empty)
    torch.cuda.synchronize()
    assert torch.equal(got_rho, want_rho) and torch.equal(got_over, want_over)
    fixed = f.cpu().numpy()
    half = got_rho.cpu().numpy()[:gr.nbx, :gr.nby]
    assert np.array_equal(half, fixed)                           # no charge: the density is the fixed map
    assert np.array_equal(got_over.cpu().numpy(), np.maximum(fixed - np.float32(gr.target), 0).astype(np.float32))
