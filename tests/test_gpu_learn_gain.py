"""What the trained learned start gains over the plain start, on netlists it has not seen: four held-out seeds of the
training generator (5,000-50,000 cells, 5-30 macros; training used seeds 0-1999, validation 100000-100031). For
each, the plain two-level placement (the reference's start) and the one from the network's proposal, both with the
tensor-core field, both to the stop. The learned start must converge on every netlist, take fewer iterations on
average (the iteration counts are deterministic; times are reported by bench.py), and keep the exact HPWL within
1.5 % of the plain start's on average."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_learned_start_gains_on_held_out_netlists():
    from autoplace_gb300 import learn
    assert os.path.exists(learn.MODEL_FILE), "the trained model is part of the package"
    model = learn.load_model()
    ls = float(model.get("lam_scale", 1.0))
    rows = learn.evaluate_start(range(200_000, 200_004), model, [ls])
    k = "learned_%g" % ls
    its = [r[k]["iters"] / r["plain"]["iters"] for r in rows]
    hp = [r[k]["hpwl"] / r["plain"]["hpwl"] for r in rows]
    tm = [r[k]["seconds"] / r["plain"]["seconds"] for r in rows]
    print("learned start: iterations / plain %s (mean %.3f), hpwl / plain %s (mean %.4f), time / plain mean %.3f"
          % (np.round(its, 3).tolist(), np.mean(its), np.round(hp, 4).tolist(), np.mean(hp), np.mean(tm)))
    assert all(r[k]["reason"] == "converged" for r in rows)
    assert np.mean(its) < 0.95
    assert np.mean(hp) <= 1.015
