"""Batches of uneven instances in one CUDA graph per phase (autoplace_gb300/batch.py, gp103_batch_*): every instance
ends exactly where its own Placer.run ends (the same kernels in the same order: positions bit for bit, the same stop
and iterations), and the autotuner's choices are valid launches that place as well."""
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
