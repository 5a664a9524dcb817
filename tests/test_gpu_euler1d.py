"""GPU: 1D Euler blocks (apps/Sod_shock_tube/Sod_shock_tube.py: LLFTeno(5), RoeAverage; apps/shu_osher/
shu_osher.py: LLFWeno(5, 'Z'), RoeAverage), FP64, with the reference's own 1D eigensystem.

* GPU vs the reference's generated code (golden fixtures ref_sod: 200 points, 200 steps; ref_shu_osher:
  400 points, 200 steps at dt = 2e-3): Sod <= 1e-12; Shu-Osher within WENO-Z's rounding floor (the
  oracle itself is 3.7e-9 from that code: eps = 1e-14 divides by (beta + eps)^2 in flat fields).
* GPU vs the oracle for the other schemes and the simple average <= 1e-12; the right-hand side <= 1e-11.
* Graph replay and eager launches give bitwise equal states.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import sod_plan, shu_osher_plan
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu

INNER = (slice(None), slice(4, -4))


def golden(case):
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_%s.npz" % case))
    return d["q0"], d["q"], int(d["n"][0]), int(d["steps"]), json.loads(str(d["params"]))


def run_gpu(plan, q0, steps):
    s = Solver(plan)
    s.set_state64_padded(q0, 4)
    s.step(steps, plan.dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def rel_err(a, b):
    return [float(np.abs(a[v] - b[v]).max() / np.abs(b[v]).max()) for v in range(b.shape[0])]


@pytest.mark.parametrize("case,make,tol", [("sod", sod_plan, 1e-12), ("shu_osher", shu_osher_plan, 1e-7)])
def test_euler1d_fp64_matches_reference_golden(case, make, tol):
    q0, q_ref, n0, steps, params = golden(case)
    plan = make(n0, dt=params["dt"])
    q = run_gpu(plan, q0, steps)
    assert max(rel_err(q, q_ref[INNER])) <= tol, rel_err(q, q_ref[INNER])
    assert max(rel_err(q0[INNER], q_ref[INNER])) > 0.1  # the waves moved


@pytest.mark.parametrize("conv,averaging", [("weno5js", "roe"), ("teno6", "roe"), ("teno5", "simple")])
def test_euler1d_fp64_matches_oracle(conv, averaging):
    q0, _, n0, _, params = golden("sod")
    plan = sod_plan(n0, dt=params["dt"], conv=conv, averaging=averaging)
    q = run_gpu(plan, q0, 100)
    q_or = O.run1d(plan, q0, 100)[INNER]
    assert max(rel_err(q, q_or)) <= 1e-12, rel_err(q, q_or)


def test_euler1d_residual_and_graph():
    q0, q_ref, n0, steps, params = golden("sod")
    plan = sod_plan(n0, dt=params["dt"])
    r_or = O.residual1d(plan, q_ref)
    s = Solver(plan)
    s.set_state64_padded(q_ref, 4)
    r = s.residual().cpu().numpy()
    s.close()
    err = [float(np.abs(r[v] - r_or[v]).max() / np.abs(r_or[v]).max()) for v in range(3)]
    assert max(err) <= 1e-11, err
    a = run_gpu(plan, q0, 7)
    b = run_gpu(plan.replace(use_graphs=False), q0, 7)
    assert np.array_equal(a, b)
