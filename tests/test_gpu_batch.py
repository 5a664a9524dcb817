"""GPU: batched ensembles (osb_batch_*, opensbli_gb300.batch.Ensemble) against single-plan runs and
the oracle.

Every instance of a batch must end where its own Solver run ends (FP64: within 1e-13, the same
arithmetic in a different launch shape; both within 1e-12 of the oracle), for uneven sizes
(including non-cubic and sizes that do not fill tiles), mixed schemes and per-instance time steps.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from opensbli_gb300.batch import Ensemble, tgv_ensemble
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import OSBError, Solver
from helpers import oracle_cfg, rel_err

pytestmark = pytest.mark.gpu


def cases(precision):
    return [tgv_plan(16, conv="weno5js", Minf=1.25, precision=precision),
            tgv_plan((20, 18, 14), precision=precision),
            tgv_plan(24, precision=precision),
            tgv_plan((33, 17, 21), conv="weno5js", Minf=1.25, precision=precision),
            tgv_plan(12, precision=precision, visc="none"),
            tgv_plan(20, conv="weno5js", Minf=1.25, precision=precision, visc="none")]


def single(plan, q0, steps, dt):
    s = Solver(plan)
    s.set_state64(q0)
    for d in range(3):
        if plan.conv == "weno5js":
            s.set_weno_shape(d, "march4", 48)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_runs(precision):
    plans = cases(precision)
    dts = [2e-3 * (1 + 0.1 * i) for i in range(len(plans))]
    q0s = [O.tgv_init(oracle_cfg(p)) for p in plans]
    ens = Ensemble(plans)
    for i, q in enumerate(q0s):
        ens.set_state64(i, q)
    ens.set_dt(dts)
    ens.step(3)
    ens.step(2)  # odd then even step count: both graphs, both buffer parities
    tol = 1e-13 if precision == "fp64" else 1e-6
    for i, p in enumerate(plans):
        qb = ens.state64(i).cpu().numpy()
        qs = single(p, q0s[i], 5, dts[i])
        assert max(rel_err(qb, qs)) <= tol, (i, rel_err(qb, qs))
        if precision == "fp64":
            cfg = oracle_cfg(p, dt=dts[i])
            assert max(rel_err(qb, O.run(cfg, q0s[i], 5))) <= 1e-12
    assert ens.launch_count() > 0
    ens.close()


def test_batch_autotune_keeps_states():
    plans = cases("fp64")
    q0s = [O.tgv_init(oracle_cfg(p)) for p in plans]
    ens = Ensemble(plans)
    for i, q in enumerate(q0s):
        ens.set_state64(i, q)
    ens.set_dt([2e-3] * len(plans))
    ens.step(1)
    best = ens.autotune(reps=1)
    assert set(best) == {"weno_x", "weno_y", "weno_z", "central"}
    assert best["central"][0] in (8, 16) and best["central"][1] in (8, 16, 32)
    for name in ("weno_x", "weno_y", "weno_z"):
        assert best[name][0] in ("march4", "march8") and best[name][1] > 0
    ens.step(2)
    for i, p in enumerate(plans):
        cfg = oracle_cfg(p, dt=2e-3)
        assert max(rel_err(ens.state64(i).cpu().numpy(), O.run(cfg, q0s[i], 3))) <= 1e-12
    ens.close()


def test_batch_needs_time_steps_and_rejects_other_plans():
    ens = Ensemble([tgv_plan(16), tgv_plan(20)])
    with pytest.raises(OSBError):
        ens.step(1)
    ens.close()
    with pytest.raises(NotImplementedError):
        Ensemble([tgv_plan(16), tgv_plan(16).replace(bc=(("symmetry", "symmetry"),) * 3)])
    with pytest.raises(OSBError):
        Ensemble([tgv_plan(16), tgv_plan(16, precision="mixed")])


def test_tgv_ensemble_runs():
    plans, states, dts = tgv_ensemble(count=12, sizes=(16, 24, 32), precision="mixed", seed=3)
    ens = Ensemble(plans)
    for i, q in enumerate(states):
        ens.set_state64(i, q)
    ens.set_dt(dts)
    ens.autotune(reps=1)
    ens.step(4)
    for i in range(len(plans)):
        q = ens.state64(i)
        assert torch.isfinite(q).all()
    ens.close()
