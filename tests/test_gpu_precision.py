"""The field's precision on a real run of the 200,000-cell netlist (200,000 cells, 210,000 nets, 20 macros over 15 % of
the region, target density 0.9, force grid 512 x 512): one level of the cells in each field mode, the field of every
16th density pass against float64 (oracle/precision.py) beside the reference's float32 FFT formula on the same map,
and the final HPWL / overflow of each mode. Bars (of the float64 field's largest value, at every checked pass):
bf16x6 1e-6, f16x3 1.5e-6, bf16x3 3e-5, fp32 (CUDA cores, float32 sums of 16 products added to a running sum)
1e-6 -- the reference's own float32 FFT formula measures up to 2e-6 on the same maps; every mode converges, its HPWL
within 0.5 % of bf16x6's."""
import json

import numpy as np
import pytest

from autoplace_gb300 import problem, synth
from oracle import precision as X

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# f16x3's two float16 terms are exact to 2^-22 of their 64-wide chunk's largest value, bf16x6's three bf16 terms to
# 2^-24 of each value: bf16x6 holds the 1e-6 bar at every pass, f16x3 (the faster default) 1.5e-6
MODES = [("f16x3", 1.5e-6), ("bf16x6", 1e-6), ("bf16x3", 3e-5), ("tf32x3", 1e-6), ("fp32", 1e-6)]


@pytest.fixture(scope="module")
def c1():
    nl, o = synth.preset("c1", seed=0)
    prob = problem.Problem(nl, problem.options(**o))
    pos0 = synth.init_positions(nl, prob.num_nodes, seed=0)
    return prob, pos0


@pytest.fixture(scope="module")
def runs(c1):
    from autoplace_gb300.engine import Placer
    prob, pos0 = c1
    out = {}
    for mode, _ in MODES:
        pl = Placer(prob, field=mode)
        r, rows = X.run_with_errors(pl, pos0, every=16)
        h, o = pl.evaluate(r["pos"])
        out[mode] = dict(reason=r["reason"], iters=r["iters"], hpwl=h, overflow=o, rows=rows)
        del pl
    summary = {m: {"iters": v["iters"], "reason": v["reason"], "hpwl": v["hpwl"], "overflow_exact": v["overflow"],
                   "field_err_max": max(r["mode_err"] for r in v["rows"]),
                   "field_err_median": float(np.median([r["mode_err"] for r in v["rows"]])),
                   "energy_err_max": max(r["mode_energy_err"] for r in v["rows"]),
                   "fft32_err_max": max(r["fft32_err"] for r in v["rows"]),
                   "fft32_energy_err_max": max(r["fft32_energy_err"] for r in v["rows"]),
                   "steps_checked": len(v["rows"])} for m, v in out.items()}
    print("c1 precision:", json.dumps(summary))
    for m, v in out.items():
        print("c1 per pass %s:" % m, json.dumps([(r["pass"], round(r["mode_err"], 9)) for r in v["rows"]]))
    return out


@pytest.mark.parametrize("mode,tol", MODES)
def test_field_error_every_checked_pass(runs, mode, tol):
    rows = runs[mode]["rows"]
    assert len(rows) >= 10
    worst = max(r["mode_err"] for r in rows)
    assert worst <= tol, (mode, worst)


def test_every_mode_converges_to_the_same_placement_quality(runs, c1):
    prob, _ = c1
    ref = runs["bf16x6"]["hpwl"]
    for mode, _ in MODES:
        r = runs[mode]
        assert r["reason"] == "converged", (mode, r["reason"])
        assert abs(r["hpwl"] - ref) <= 0.005 * ref, (mode, r["hpwl"], ref)
