"""The learned start's kernels (csrc/learn.cu) against the CPU oracle (oracle/learn_ref.py): the cluster features
against their numpy statement, the network's forward pass and every parameter gradient against torch autograd on the
CPU (bf16-rounded weights, fp32 arithmetic in both), and training that lowers the loss."""
import numpy as np
import pytest

from autoplace_gb300 import problem, synth
from oracle import learn_ref as R

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda"


@pytest.fixture(scope="module")
def clusters():
    """A 12,000-cell netlist with 12 macros, clustered on the device as a placement clusters it."""
    from autoplace_gb300 import cluster
    nl = synth.make_netlist(12000, 12600, window=150, macros=12, cover=0.12, fixed_pin_share=0.02, seed=21)
    prob = problem.Problem(nl, problem.options(target_density=0.9, num_bin=0, cluster_ratio=5.0, seed=21))
    coarse = cluster.coarse_problem(prob, device=DEV)
    torch.cuda.synchronize()
    cs = coarse.problem.csr
    host = lambda a: a.cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    arrays = dict(net_start=host(cs.net_start), pin_cell=host(cs.cell32), pin_off=host(cs.off),
                  cell_start=host(cs.cell_start), cell_pin=host(cs.cell_pin))
    return prob, coarse, arrays


def test_features_match_oracle(clusters):
    from autoplace_gb300 import learn
    prob, coarse, a = clusters
    g, x = learn.cluster_inputs(coarse, prob, DEV)
    x = x.cpu().numpy()
    K = coarse.num
    area = np.asarray(coarse.problem.node_size[:K], np.float64).prod(1)
    pins = np.bincount(coarse.cid, weights=np.asarray(prob.nl.cell_pins, np.float64), minlength=K)
    ref = R.features(a["net_start"], a["pin_cell"], a["pin_off"], a["cell_start"], a["cell_pin"], K, area, pins,
                     prob.nl.width, prob.nl.height)
    assert x.shape == ref.shape == (K, 10)
    # (the 64 harmonic sweeps run in float32 on the device: 1e-4 there, 1e-5 on the rest)
    assert np.abs(x[:, :8] - ref[:, :8]).max() <= 1e-5, np.abs(x - ref).max(0)
    assert np.abs(x[:, 8:] - ref[:, 8:]).max() <= 1e-4, np.abs(x - ref).max(0)
    anchored = ref[:, 6] > 0
    assert 0.5 < anchored.mean() <= 1.0                      # most clusters reach a fixed pin within 12 hops


def test_forward_and_gradients_match_autograd(clusters):
    from autoplace_gb300 import learn
    prob, coarse, a = clusters
    g, x = learn.cluster_inputs(coarse, prob, DEV)
    K = coarse.num
    params = learn.init_params(seed=3)
    rng = np.random.default_rng(4)
    for k in params:                                         # non-zero biases too
        if k[0] == "b":
            params[k] = (rng.standard_normal(params[k].shape) * 0.1).astype(np.float32)
    target = rng.random((K, 2)).astype(np.float32)
    net = learn.Net(params, device=DEV)
    work = learn.Pass.for_graph(net, g)
    t = torch.as_tensor(target).to(DEV)
    loss = float(work.loss_and_grad(g, x, t).cpu())
    y = work.y[:K].cpu().numpy()
    torch.cuda.synchronize()
    ry, rloss, rgrads = R.forward_backward(params, x.cpu().numpy(), target, a["net_start"], a["pin_cell"],
                                           a["cell_start"], a["cell_pin"], K)
    assert np.abs(y - ry).max() <= 1e-5
    assert abs(loss - rloss) <= 1e-5 * rloss
    for name, rg in rgrads.items():
        gg = net.gviews[name].cpu().numpy()
        err = np.abs(gg - rg).max() / max(np.abs(rg).max(), 1e-12)
        assert err <= 1e-4, (name, err)


def test_training_lowers_the_loss(clusters):
    """Adam on one graph with a learnable target (each cluster's propagated anchor, one of its features, kept off the
    region's edge): the loss falls by 5x in 300 steps."""
    from autoplace_gb300 import learn
    prob, coarse, a = clusters
    g, x = learn.cluster_inputs(coarse, prob, DEV)
    target = torch.clamp(x[:, 3:5], 0.05, 0.95).contiguous()
    net = learn.Net(learn.init_params(seed=0), device=DEV)
    work = learn.Pass.for_graph(net, g)
    first = float(work.loss_and_grad(g, x, target).cpu())
    for _ in range(300):
        work.loss_and_grad(g, x, target)
        net.adam(3e-3, g.stream)
    last = float(work.loss_and_grad(g, x, target).cpu())
    assert last < first / 5, (first, last)
