"""GPU: TENO with the cut-off adapted by the modified Ducros sensor on 3D blocks
(schemes/spatial/teno.py:430-443, schemes/spatial/shock_sensors.py:12-49).

* FP64 GPU vs the reference's own generated code (golden fixture ref_tgv_teno_adaptive: TENO5,
  16^3, Minf 1.25, 10 steps) <= 1e-12, max-normalised per conserved variable.
* The per-point cut-off (the reference's TENO_B0 field) equals the oracle's bit for bit on a state
  where the sensor takes every level 10^-6 .. 10^-10.
* FP64 GPU vs the oracle for TENO5 and TENO6 on a non-cubic grid, from a perturbed state, for
  every launch shape of the flux kernels (each reads the cut-off at its own index) <= 1e-12.
* Graph replay and eager launches give bitwise equal states; mixed precision stays within 1e-5
  (relative L2) of the FP64 oracle.
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


def perturbed(cfg, amp, seed=3):
    """Taylor-Green state with random velocity perturbations: compressions and rotations of
    comparable size, so that the sensor spreads over [0, 1]."""
    q = O.tgv_init(cfg)
    rng = np.random.default_rng(seed)
    for c in range(3):
        q[1 + c] += amp * q[0] * rng.standard_normal(q[0].shape)
    return q


def test_adaptive_fp64_matches_reference_golden():
    q_ref, n, steps, params = load_golden("tgv_teno_adaptive")
    plan = golden_plan("tgv_teno_adaptive", n=n).replace(Minf=params["Minf"])
    assert plan.teno_adaptive and plan.conv == "teno5"
    cfg = oracle_cfg(plan, dt=params["dt"])
    q = run_gpu(plan, O.tgv_init(cfg), steps, params["dt"])
    err = rel_err(q, q_ref)
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adaptive_cutoff_field_matches_oracle(precision):
    plan = tgv_plan((20, 24, 18), conv="teno5", Minf=1.25).replace(teno_adaptive=True, precision=precision)
    cfg = oracle_cfg(plan, dt=2e-3)
    q = perturbed(cfg, 0.05)
    ct_or = O.cutoff(cfg, q)
    s = Solver(plan)
    s.set_state64(q)
    ct = s.teno_cutoff().cpu().numpy()
    s.close()
    assert len(np.unique(ct_or)) == 5
    if precision == "fp64":
        assert np.array_equal(ct, ct_or), int((ct != ct_or).sum())
    else:
        # the cut-off is held in the state precision (10^-k rounded to FP32), and the FP32 sensor may
        # move a point whose exponent lies within rounding of an integer to the next level
        ct_or32 = ct_or.astype(np.float32).astype(np.float64)
        assert set(np.unique(ct)) <= set(np.unique(ct_or32)) and (ct != ct_or32).mean() < 1e-2


@pytest.mark.parametrize("conv", ["teno5", "teno6"])
@pytest.mark.parametrize("shapes", [
    None,
    (("tile", 32), ("tile", 32), ("tile", 32)),
    (("march8", 16), ("march8", 24), ("march8", 20)),
    (("march4", 48), ("march4", 7), ("march4", 9)),
])
def test_adaptive_fp64_matches_oracle_all_shapes(conv, shapes):
    plan = tgv_plan((20, 24, 18), conv=conv, Minf=1.25).replace(teno_adaptive=True)
    dt = 1e-3
    cfg = oracle_cfg(plan, dt=dt)
    q0 = perturbed(cfg, 0.02)
    q_or = O.run(cfg, q0, 3)
    q = run_gpu(plan, q0, 3, dt, shapes)
    err = rel_err(q, q_or)
    assert max(err) <= 1e-12, err
    # the perturbation makes the adaptive cut-off differ from the fixed one
    q_fix = O.run(oracle_cfg(plan.replace(teno_adaptive=False), dt=dt), q0, 3)
    assert max(rel_err(q_fix, q_or)) > 1e-9


def test_adaptive_graph_matches_eager_and_mixed_error():
    q_ref, n, steps, params = load_golden("tgv_teno_adaptive")
    plan = golden_plan("tgv_teno_adaptive", n=n).replace(Minf=params["Minf"])
    cfg = oracle_cfg(plan, dt=params["dt"])
    q0 = O.tgv_init(cfg)
    qg = run_gpu(plan, q0, 4, params["dt"])
    qe = run_gpu(plan.replace(use_graphs=False), q0, 4, params["dt"])
    assert np.array_equal(qg, qe)
    qm = run_gpu(plan.replace(precision="mixed"), q0, steps, params["dt"])
    l2 = rel_l2(qm[[0, 1, 2, 4]], q_ref[[0, 1, 2, 4]])
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2


def test_cutoff_needs_an_adaptive_plan():
    s = Solver(tgv_plan(16, conv="teno5", Minf=1.25))
    s.init_tgv()
    with pytest.raises(Exception):
        s.teno_cutoff()
    s.close()
