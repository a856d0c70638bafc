"""Batches of uneven instances in one CUDA graph (autoplace_gb300/batch.py, gp103_batch_*): every instance ends
exactly where its own Placer.run ends (the same kernels in the same order: positions bit for bit, the same stop and
iterations), the level's set-up and the hand-over between the phases, made on the device, give the state of the
host's statement of the rules bit for bit, and the autotuner's choices are valid launches that place as well."""
import math

import numpy as np
import pytest

from autoplace_gb300 import problem, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def instances():
    probs, pos = [], []
    for nl, o in synth.batch_instances(count=6, seed=3, lo=3000, hi=30000):
        p = problem.Problem(nl, problem.options(**o))
        probs.append(p)
        pos.append(synth.init_positions(nl, p.num_nodes, seed=1))
    return probs, pos


def test_batch_matches_one_by_one(instances):
    from autoplace_gb300.batch import Batch
    from autoplace_gb300.engine import Placer
    probs, pos = instances
    assert len({p.force.nbx for p in probs}) >= 2                 # uneven grids
    b = Batch(probs)
    res, per, wall = b.run(pos)
    assert np.all(per > 0) and np.all(per <= wall + 1e-3)
    for p, p0, r in zip(probs, pos, res):
        ref = Placer(p).run(p0)
        assert r["reason"] == ref["reason"] and r["iters"] == ref["iters"], (r["reason"], r["iters"], ref["iters"])
        assert np.array_equal(r["pos"].cpu().numpy().view(np.uint32), ref["pos"].cpu().numpy().view(np.uint32))
    # the graphs are kept: a second run of the same batch gives the same placements
    res2, _, _ = b.run(pos)
    for r, r2 in zip(res, res2):
        assert np.array_equal(r["pos"].cpu().numpy(), r2["pos"].cpu().numpy())


@pytest.mark.parametrize("lam0", [0.0, 1e-4])
def test_set_up_matches_the_host_rule(instances, lam0):
    """gp103_begin against the probe steps stated on the host (src/nesterov_optimizer.py:56-63 and :15-32: a probe of
    --lr, the step length from it, the gradient again, u = v, the optimiser's probe), for a fresh run (the start's T)
    and a resumed one (the density phase's S), bit for bit."""
    from autoplace_gb300.engine import Placer, SK, S_FIELDS, TI
    from autoplace_gb300.native import T_SIZE
    probs, pos = instances
    for p, p0 in list(zip(probs, pos))[:2]:
        pl = Placer(p, use_graphs=False)
        gam, o = pl.start_gamma, p.opts
        pl.load(p0)
        with torch.cuda.stream(pl.stream):
            pl.kp.copy_(torch.tensor([gam, lam0, lam0, 0, 0], dtype=torch.float32))
            pl.cur.zero_()
        v, g, probe, g2 = pl.V[0], pl.G[0], pl.tmp[0], pl.tmp[1]
        w, pc = (lam0, lam0) if lam0 > 0 else (0.0, -1.0)
        pl.eval(v, g, weight=w, precond=pc)
        d1 = pl.probe(v, g, o.lr, probe)
        d2 = pl.eval(probe, g2, g_ref=g, weight=w, precond=pc)[0]
        lr = math.sqrt(d1) / math.sqrt(d2)
        pl.eval(v, g, weight=w, precond=pc)
        d1 = pl.probe(v, g, lr, probe)
        d2 = pl.eval(probe, g2, g_ref=g, weight=w, precond=pc)[0]
        alpha = math.sqrt(d1) / math.sqrt(d2)
        g_host = g.cpu().numpy().copy()
        with torch.cuda.stream(pl.stream):
            for t in (pl.T, pl.S, pl.kp, pl.U[0], pl.G[0], pl.best):
                t.zero_()
            pl.cur.fill_(1)
        resume = dict(lam=lam0, gam=gam, iter=7, first_iter=3, hpwl=123.5) if lam0 > 0 else None
        ctx = pl.begin(p0, resume)
        pl.sync()
        assert ctx["start"] == (lam0 == 0) and int(pl.cur.cpu()) == 0
        if lam0 == 0:
            T = np.zeros(T_SIZE)
            T[TI["alpha"]], T[TI["a"]], T[TI["start_tol"]], T[TI["inner"]] = alpha, 1.0, o.start_tol, o.inner_iter
            assert np.array_equal(pl.T.cpu().numpy().view(np.uint64), T.view(np.uint64))
            kp = np.array([gam, 0, 0, alpha, 0], dtype=np.float32)
        else:
            S = np.zeros(len(S_FIELDS))
            S[SK["lam"]], S[SK["gam"]], S[SK["alpha"]], S[SK["a"]] = lam0, gam, alpha, 1.0
            S[SK["iter"]], S[SK["hpwl_prev"]], S[SK["mu"]], S[SK["loop_it"]] = 7, 123.5, 1.0, 3
            S[SK["best_hpwl"]] = S[SK["best_ovf"]] = math.inf
            assert np.array_equal(pl.S.cpu().numpy().view(np.uint64), S.view(np.uint64))
            kp = np.array([gam, lam0, lam0, alpha, 0], dtype=np.float32)
            assert np.array_equal(pl.best.cpu().numpy(), v.cpu().numpy())
        assert np.array_equal(pl.kp.cpu().numpy().view(np.uint32), kp.view(np.uint32))
        assert np.array_equal(pl.U[0].cpu().numpy(), v.cpu().numpy())
        assert np.array_equal(pl.G[0].cpu().numpy().view(np.uint32), g_host.view(np.uint32))


def test_hand_over_matches_the_host_rule(instances):
    """gp103_start_to_density against the rule stated on the host in float64 (src/run_placement.py:60-64: density
    weight x tension unit; src/gpu_loop.py:38-48: the density phase's state, kp with the Nesterov coefficient)."""
    from autoplace_gb300 import native
    from autoplace_gb300.engine import Placer, SK, S_FIELDS, TI
    probs, pos = instances
    for p, p0 in list(zip(probs, pos))[:3]:
        pl = Placer(p, use_graphs=False)
        ctx = pl.begin(p0)
        while True:
            pl._replay(native.PHASE_START)
            pl.sync()
            Th = pl.T.cpu().numpy()
            if Th[TI["done"]] or Th[TI["stop"]]:
                break
        assert pl.start_over(ctx, Th) is None
        cur = int(pl.cur.cpu())
        lam = p.opts.density_weight * pl.tension_unit(pl.V[cur])[0]
        a = Th[TI["a"]]
        coef = (a - 1) / ((1 + math.sqrt(4 * a * a + 1)) / 2)
        S = np.zeros(len(S_FIELDS))
        S[SK["lam"]], S[SK["gam"]], S[SK["alpha"]], S[SK["a"]] = lam, pl.start_gamma, Th[TI["alpha"]], a
        S[SK["iter"]], S[SK["hpwl_prev"]], S[SK["mu"]] = Th[TI["iter"]], Th[TI["hpwl"]], 1.0
        S[SK["best_hpwl"]] = S[SK["best_ovf"]] = math.inf
        S[SK["loop_it"]] = ctx["start_iters"]
        kp = np.array([pl.start_gamma, lam, lam, Th[TI["alpha"]], coef], dtype=np.float32)
        with torch.cuda.stream(pl.stream):
            pl.best.zero_()
        pl.hand_over(ctx)
        pl.sync()
        assert np.array_equal(pl.S.cpu().numpy().view(np.uint64), S.view(np.uint64))
        assert np.array_equal(pl.kp.cpu().numpy().view(np.uint32), kp.view(np.uint32))
        assert np.array_equal(pl.best.cpu().numpy().view(np.uint32), pl.V[cur].cpu().numpy().view(np.uint32))


def test_tuned_batch_places_as_well(instances):
    """Tuned per instance (field mode, WA lane groups): each instance converges, its HPWL within 1 % of the default
    settings' (a different lane partition sums in a different order)."""
    from autoplace_gb300 import tune
    from autoplace_gb300.batch import Batch
    from autoplace_gb300.engine import Placer
    probs, pos = instances
    tuned = [tune.tune(p, p0) for p, p0 in zip(probs, pos)]
    for t in tuned:
        assert t["field"] in ("f16x3", "fp32") and t["wa"] in tune.WA_CHOICES and t["ms_per_pass"] > 0
    res, _, _ = Batch(probs, tuned=tuned).run(pos)
    for p, p0, r in zip(probs, pos, res):
        ref = Placer(p).run(p0)
        assert r["reason"] == "converged"
        h = Placer(p).evaluate(r["pos"])[0]
        hr = Placer(p).evaluate(ref["pos"])[0]
        assert abs(h - hr) <= 0.01 * hr
