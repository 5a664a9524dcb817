"""GPU: Solver.advance_host_states, the pipelined advance of independent states held in pinned host
memory, gives bitwise the results of advancing each state on its own (set_state64, step, state64)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt
from opensbli_gb300.runtime import Solver
from helpers import oracle_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_advance_host_states_matches_one_by_one(precision):
    plan = tgv_plan((24, 20, 16), conv="weno5js", Minf=1.25, precision=precision)
    dt = tgv_cfl_dt(plan)
    q0 = O.tgv_init(oracle_cfg(plan, dt=dt))
    rng = np.random.default_rng(0)
    inputs = []
    for k in range(5):  # five different states: the TGV field with seeded momentum noise
        q = q0.copy()
        q[1:4] += 1e-3 * rng.standard_normal(q[1:4].shape)
        inputs.append(torch.from_numpy(q).pin_memory())
    outputs = [torch.empty_like(inputs[0]).pin_memory() for _ in inputs]
    s = Solver(plan)
    s.advance_host_states(inputs, outputs, dt, nsteps=2)
    for q_in, q_out in zip(inputs, outputs):
        s.set_state64(q_in.to(s.device))
        s.step(2, dt)
        assert torch.equal(s.state64().cpu(), q_out)
    s.close()
