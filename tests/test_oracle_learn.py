"""CPU checks of the learned start's oracle (oracle/learn_ref.py) and host logic: the autograd gradients against
central differences (float64 would be exact; the oracle runs fp32, so the check is at fp32 precision), the anchor
propagation of the features on a hand-made graph, and the model file round trip."""
import numpy as np
import pytest

from oracle import learn_ref as R

torch = pytest.importorskip("torch")


def _tiny_graph():
    """4 clusters, 4 nets: net 0 (c0, c1, fixed pin at (10, 20)), net 1 (c1, c2), net 2 (c2, c3), net 3 (c0, c3)."""
    net_start = np.array([0, 3, 5, 7, 9])
    pin_cell = np.array([0, 1, 4, 1, 2, 2, 3, 0, 3])            # cell 4 = K: the fixed pin
    pin_off = np.zeros((9, 2), np.float32)
    pin_off[2] = [10.0, 20.0]
    cell_pin = np.array([0, 7, 1, 3, 4, 5, 6, 8])                # the movable pins by cell, in pin order
    cell_start = np.array([0, 2, 4, 6, 8])
    return net_start, pin_cell, pin_off, cell_start, cell_pin


def test_features_anchor_propagation():
    ns, pc, po, cs, cp = _tiny_graph()
    f = R.features(ns, pc, po, cs, cp, 4, np.ones(4), np.full(4, 2.0), 100.0, 100.0, max_hop=4, sweeps=200)
    # clusters 0 and 1 sit on the fixed pin's net: anchored at hop 0 at (0.1, 0.2); 2 and 3 reach it at hop 1
    assert np.allclose(f[:, 3], 0.1) and np.allclose(f[:, 4], 0.2)
    assert np.allclose(f[:, 5], [0.0, 0.0, 0.25, 0.25]) and np.all(f[:, 6] == 1.0)
    assert np.allclose(f[:, 0], 0.0) and np.allclose(f[:, 1], np.log1p(2) / 4)
    # the harmonic coordinates of a graph with one fixed pin converge to that pin's position
    assert np.allclose(f[:, 8], 0.1, atol=1e-6) and np.allclose(f[:, 9], 0.2, atol=1e-6)


def test_autograd_against_central_differences():
    import autoplace_gb300.learn as L
    ns, pc, po, cs, cp = _tiny_graph()
    rng = np.random.default_rng(0)
    params = L.init_params(seed=1)
    for k in params:
        params[k] = (params[k] + rng.standard_normal(params[k].shape) * 0.05).astype(np.float32)
    x = rng.random((4, 10)).astype(np.float32)
    t = rng.random((4, 2)).astype(np.float32)
    y, loss, grads = R.forward_backward(params, x, t, ns, pc, cs, cp, 4)
    # biases are not rounded to bf16: central differences on them in float64 arithmetic of the same forward
    for name in ("bo", "b1", "b3"):
        g = grads[name]
        k = int(np.argmax(np.abs(g)))
        h = 1e-2
        up, dn = dict(params), dict(params)
        up[name] = params[name].copy().astype(np.float64)
        dn[name] = params[name].copy().astype(np.float64)
        up[name].flat[k] += h
        dn[name].flat[k] -= h
        lu = R.forward_backward({a: np.asarray(b, np.float32) for a, b in up.items()}, x, t, ns, pc, cs, cp, 4)[1]
        ld = R.forward_backward({a: np.asarray(b, np.float32) for a, b in dn.items()}, x, t, ns, pc, cs, cp, 4)[1]
        fd = (lu - ld) / (2 * h)
        assert abs(fd - g.flat[k]) <= 2e-3 * max(abs(g.flat[k]), 1e-3), (name, fd, g.flat[k])


def test_model_file_round_trip(tmp_path):
    import autoplace_gb300.learn as L
    p = L.init_params(seed=2)
    path = str(tmp_path / "m.npz")
    L.save_model(path, p, lam_scale=3.0, epochs=7)
    m = L.load_model(path)
    assert m["lam_scale"] == 3.0 and m["epochs"] == 7
    assert set(m["params"]) == set(p) and all(np.array_equal(m["params"][k], p[k]) for k in p)
