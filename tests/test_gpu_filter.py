"""GPU: the WENO5 non-linear filter (filters/WENO_filter.py, dissipation_sensor='Constant') applied
after every full RK3 step of the central skew-symmetric Taylor-Green scheme.

* FP64 GPU vs the reference's own generated code (golden fixture ref_tgv_filter: 16^3, Minf 1.25,
  10 steps) <= 1e-12, max-normalised per conserved variable.
* FP64 GPU vs the oracle on a non-cubic grid for every launch shape of the filter's flux passes
  (tiled, line-marching with 4 and 8 lines per block) <= 1e-12.
* Graph replay and eager launches give bitwise equal states; mixed precision stays within 2e-6
  (relative L2) of the FP64 oracle after 5 steps.
"""
import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver
from helpers import golden_plan, load_golden, oracle_cfg, rel_err, rel_l2

pytestmark = pytest.mark.gpu


def run_gpu(plan, q0, steps, dt, shapes=None):
    s = Solver(plan)
    if shapes:
        for d, (kind, seg) in enumerate(shapes):
            s.set_weno_shape(d, kind, seg)
    s.set_state64(q0)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def test_filter_fp64_matches_reference_golden():
    q_ref, n, steps, params = load_golden("tgv_filter")
    plan = golden_plan("tgv_filter", n=n).replace(Minf=params["Minf"])
    assert plan.filter == "weno5_constant" and plan.conv == "central_skew"
    cfg = oracle_cfg(plan, dt=params["dt"])
    q = run_gpu(plan, O.tgv_init(cfg), steps, params["dt"])
    err = rel_err(q, q_ref)
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("shapes", [
    None,
    (("tile", 32), ("tile", 32), ("tile", 32)),
    (("march8", 16), ("march8", 24), ("march8", 20)),
    (("march4", 48), ("march4", 7), ("march4", 9)),
])
def test_filter_fp64_matches_oracle_all_shapes(shapes):
    n = (20, 24, 18)
    plan = tgv_plan(n, conv="central_skew", Minf=1.25).replace(filter="weno5_constant")
    dt = 2.5e-3
    cfg = oracle_cfg(plan, dt=dt)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 4)
    q = run_gpu(plan, q0, 4, dt, shapes)
    err = rel_err(q, q_or)
    assert max(err) <= 1e-12, err


def test_filter_graph_matches_eager_and_mixed_error():
    n = 24
    plan = tgv_plan(n, conv="central_skew", Minf=1.25).replace(filter="weno5_constant")
    dt = 2.5e-3
    cfg = oracle_cfg(plan, dt=dt)
    q0 = O.tgv_init(cfg)
    qg = run_gpu(plan, q0, 3, dt)
    qe = run_gpu(plan.replace(use_graphs=False), q0, 3, dt)
    assert np.array_equal(qg, qe)
    q_or = O.run(cfg, q0, 5)
    qm = run_gpu(plan.replace(precision="mixed"), q0, 5, dt)
    l2 = rel_l2(qm[[0, 1, 2, 4]], q_or[[0, 1, 2, 4]])
    assert np.isfinite(qm).all() and max(l2) <= 2e-6, l2
