"""GPU: 2D Euler blocks (apps/inviscid_shock_reflection/inviscid_shock.py): WENO5-Z with SimpleAverage,
a Dirichlet inlet, extrapolation at the outlet, a symmetry face at x1 = 0 and the shock generator's
Dirichlet face at the top, a Cartesian grid and no viscous terms.

* FP64 GPU vs the reference's own generated code (golden fixture ref_shock_reflection: 64 x 32, 30
  steps at dt = 1) within WENO-Z's rounding floor: the oracle itself agrees with that code to 1.5e-8
  (eps = 1e-14 divides by (beta + eps)^2 where a characteristic field is flat, as on the TGV and
  Katzer WENO-Z fixtures).
* FP64 GPU vs the oracle for WENO5-JS and TENO5 with SimpleAverage and for WENO5-JS with the Roe
  average <= 1e-12 on a wider block; the right-hand side <= 1e-11.
* Graph replay and eager launches give bitwise equal states; mixed precision within 1e-5 (relative L2).
* The doubly periodic density wave of apps/euler_wave/euler_wave.py (two-register RungeKutta(3)):
  FP64 vs its golden fixture and vs the oracle <= 1e-12, graph = eager, mixed within 1e-5.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import shock_reflection_plan
from opensbli_gb300.runtime import Solver, OSBError

pytestmark = pytest.mark.gpu

INNER = (slice(None), slice(4, -4), slice(4, -4))


def golden():
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_shock_reflection.npz"))
    return d["q0"], d["q"], tuple(int(x) for x in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def widen(q, n0):
    """The padded state q [4][n1+8][m0+8] extended in x0 to n0 interior points by repeating its last
    interior column (the free stream of the initial state is uniform in x0)."""
    m0 = q.shape[-1] - 8
    cols = [q[..., :4 + m0]] + [q[..., 4 + m0 - 1:4 + m0]] * (n0 - m0) + [q[..., 4 + m0:]]
    return np.concatenate(cols, axis=-1)


def run_gpu(plan, q0, steps):
    s = Solver(plan)
    s.set_state64_padded(q0, 4)
    s.step(steps, plan.dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def rel_err(a, b):
    return [float(np.abs(a[v] - b[v]).max() / np.abs(b[v]).max()) for v in range(b.shape[0])]


def test_shock_reflection_fp64_matches_reference_golden():
    q0, q_ref, n, steps, params = golden()
    plan = shock_reflection_plan(*n, dt=params["dt"])
    q = run_gpu(plan, q0, steps)
    err = rel_err(q, q_ref[INNER])
    assert max(err) <= 1e-7, err
    # the shock moved into the block: a solver that stood still could not pass
    assert max(rel_err(q0[INNER], q_ref[INNER])) > 0.1


@pytest.mark.parametrize("conv,averaging", [("weno5js", "simple"), ("teno5", "simple"), ("weno5js", "roe")])
def test_shock_reflection_fp64_matches_oracle(conv, averaging):
    q0, _, n, _, params = golden()
    q0w = widen(q0, 96)
    plan = shock_reflection_plan(96, n[1], dt=params["dt"], conv=conv, averaging=averaging)
    q_or = O.run2d(plan, q0w, 12)[INNER]
    q = run_gpu(plan, q0w, 12)
    err = rel_err(q, q_or)
    assert max(err) <= 1e-12, err


def test_shock_reflection_residual_matches_oracle():
    q0, q_ref, n, _, params = golden()
    plan = shock_reflection_plan(*n, dt=params["dt"], conv="weno5js")
    r_or = O.residual2d(plan, q_ref)
    s = Solver(plan)
    s.set_state64_padded(q_ref, 4)
    r = s.residual().cpu().numpy()
    s.close()
    scale = [np.abs(r_or[v]).max() for v in range(4)]
    err = [float(np.abs(r[v] - r_or[v]).max() / scale[v]) for v in range(4)]
    assert max(err) <= 1e-11, err


def test_shock_reflection_graph_matches_eager_and_mixed_error():
    q0, q_ref, n, steps, params = golden()
    plan = shock_reflection_plan(*n, dt=params["dt"])
    a = run_gpu(plan, q0, 5)
    b = run_gpu(plan.replace(use_graphs=False), q0, 5)
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), q0, steps)
    ref = q_ref[INNER]
    mom = float(np.linalg.norm(ref[1]))
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / (mom if v in (1, 2) else np.linalg.norm(ref[v]))) for v in range(4)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2


def test_cartesian_block_takes_no_coordinate():
    s = Solver(shock_reflection_plan(64, 32))
    with pytest.raises(OSBError, match="Cartesian"):
        s.set_coordinate(np.zeros((40, 72)), 4)
    s.close()


# ---- the doubly periodic Euler density wave (apps/euler_wave/euler_wave.py): WENO5-Z, the simple
# average, RungeKutta(3) with two registers ----

def test_euler_wave_fp64_matches_reference_golden_and_oracle():
    from opensbli_gb300.plan import euler_wave_plan
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_euler_wave.npz"))
    n = tuple(int(x) for x in d["n"])
    params = json.loads(str(d["params"]))
    plan = euler_wave_plan(*n, dt=params["dt"])
    q = run_gpu(plan, d["q0"], int(d["steps"]))
    err = rel_err(q, d["q"][INNER])
    assert max(err) <= 1e-12, err
    for conv in ("weno5js", "teno5"):
        p2 = plan.replace(conv=conv, weno_eps=1e-6)
        q_or = O.run2d(p2, d["q0"], 20)[INNER]
        assert max(rel_err(run_gpu(p2, d["q0"], 20), q_or)) <= 1e-12


def test_euler_wave_graph_matches_eager_and_mixed_error():
    from opensbli_gb300.plan import euler_wave_plan
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_euler_wave.npz"))
    n = tuple(int(x) for x in d["n"])
    plan = euler_wave_plan(*n, dt=json.loads(str(d["params"]))["dt"])
    a = run_gpu(plan, d["q0"], 6)
    b = run_gpu(plan.replace(use_graphs=False), d["q0"], 6)
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), d["q0"], int(d["steps"]))
    ref = d["q"][INNER]
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / np.linalg.norm(ref[v])) for v in range(4)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2
