"""GPU: mixed precision on 2D blocks with the characteristic flux formed in FP64 arithmetic next to
strong shocks (osb_plan_desc.shock_fp64, a pressure ratio between the interface's two points).

* Threshold 1 takes every interface with a pressure difference into FP64.  The mixed error against
  the FP64 run stays where it was (WENO5-JS on the Katzer block, 40 steps: 8.7e-8 against 8.3e-8):
  with the double-float point fluxes of the FP32 path the flux arithmetic is no longer what limits
  the mixed precision, the FP32 state is.
* A threshold no interface reaches gives the plain mixed result.
"""
import numpy as np
import pytest

from opensbli_gb300.runtime import Solver
from helpers import load_golden_2d, golden_plan_2d

pytestmark = pytest.mark.gpu


def run(plan, q0, x1, steps, dt):
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0, 4)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def l2(a, b):
    return max(float(np.linalg.norm(a[v] - b[v]) / np.linalg.norm(b[v])) for v in range(b.shape[0]))


def test_fp64_flux_next_to_shocks_runs_and_keeps_the_mixed_error():
    q0, x1, _, n, _, params = load_golden_2d("katzer_weno")
    plan = golden_plan_2d("katzer_weno", n=n).replace(dt=params["dt"])
    steps = 40
    ref = run(plan, q0, x1, steps, params["dt"])
    mixed = plan.replace(precision="mixed")
    e_off = l2(run(mixed, q0, x1, steps, params["dt"]), ref)
    e_all = l2(run(mixed.replace(shock_fp64=1.0), q0, x1, steps, params["dt"]), ref)
    assert e_all <= 2.0 * e_off and e_all < 1e-6, (e_all, e_off)
    e_none = l2(run(mixed.replace(shock_fp64=1e6), q0, x1, steps, params["dt"]), ref)
    assert abs(e_none - e_off) <= 1e-3 * e_off, (e_none, e_off)
