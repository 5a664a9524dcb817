"""GPU: the TMA plane pipeline of the fused central/RK kernel (FP32 plans with WENO fluxes) against the
register-staged loads: same arithmetic, so bitwise equal results, for both tile heights and for grids
whose tiles do not divide the domain (boxes reaching past the array read zeros that are never used)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver
from helpers import oracle_cfg

pytestmark = pytest.mark.gpu


def run(plan, q0, tma, ty, steps):
    s = Solver(plan)
    s.set_state64(q0)
    s.set_tma(tma)
    s.set_central_shape(ty)
    active = s.tma_active()
    r = s.residual().double().cpu().numpy()
    s.step(steps, 2e-3)
    q = s.state64().cpu().numpy()
    s.reduce("nancheck")  # also reports a TMA wait that gave up
    s.close()
    return active, r, q


@pytest.mark.parametrize("n", [(32, 32, 32), (45, 37, 29)])
@pytest.mark.parametrize("ty", [8, 16])
@pytest.mark.parametrize("conv", ["weno5js", "weno5z"])
def test_tma_equals_register_path(n, ty, conv):
    plan = tgv_plan(n, conv=conv, Minf=1.25, precision="mixed")
    q0 = O.tgv_init(oracle_cfg(plan))
    a_on, r_on, q_on = run(plan, q0, True, ty, 3)
    a_off, r_off, q_off = run(plan, q0, False, ty, 3)
    assert a_on and not a_off
    assert np.array_equal(r_on, r_off)
    assert np.array_equal(q_on, q_off)


def test_tma_not_used_for_fp64_or_central():
    for plan in (tgv_plan(16, conv="weno5js", Minf=1.25), tgv_plan(16, precision="mixed")):
        s = Solver(plan)
        s.init_tgv()
        assert not s.tma_active()
        s.close()
