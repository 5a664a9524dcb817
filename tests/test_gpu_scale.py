"""Full-size GPU checks at the benchmark configuration, through size-independent properties:
periodic conservation of mass, momentum and energy sums, finiteness, kinetic-energy decay, and the
mixed path against the FP64 path after a few steps."""
import math

import numpy as np
import pytest
import torch

from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_weno_256_conservation(precision):
    plan = tgv_plan(256, conv="weno5js", Minf=1.25, precision=precision)
    dt = tgv_cfl_dt(plan)
    s = Solver(plan)
    s.init_tgv()
    q0 = s.state64()
    tot0 = q0.sum(dim=(1, 2, 3))
    ke0 = s.reduce("ke")
    s.step(2, dt)
    q = s.state64()
    tot = q.sum(dim=(1, 2, 3))
    assert torch.isfinite(q).all()
    # periodic grid: the WENO flux difference and the linear central viscous terms telescope, so the
    # totals of rho and rhou_i are conserved up to roundoff (FP64 register, FP32 or FP64 fluxes); the
    # energy equation's viscous work is in expanded, non-telescoping form, so its total only
    # changes by the truncation error
    N = q.shape[1] * q.shape[2] * q.shape[3]
    tol = 1e-12 if precision == "fp64" else 1e-8
    assert abs(float(tot[0] - tot0[0])) / float(tot0[0]) < tol
    assert abs(float(tot[4] - tot0[4])) / float(tot0[4]) < 1e-6
    for v in (1, 2, 3):
        assert abs(float(tot[v] - tot0[v])) / N < (1e-12 if precision == "fp64" else 1e-7)
    assert s.reduce("ke") < ke0
    assert s.reduce("nancheck") == 0.0
    s.close()


def test_weno_128_mixed_vs_fp64():
    plan = tgv_plan(128, conv="weno5js", Minf=1.25)
    dt = tgv_cfl_dt(plan)
    out = {}
    for prec in ("fp64", "mixed"):
        s = Solver(plan.replace(precision=prec))
        s.init_tgv()
        s.step(10, dt)
        out[prec] = s.state64().cpu().numpy()
        s.close()
    for v in range(5):
        ref = out["fp64"][v]
        l2 = np.linalg.norm(out["mixed"][v] - ref) / np.linalg.norm(ref)
        assert l2 < 1e-5, (v, l2)
