"""GPU: the Cartesian 2D Navier-Stokes block of apps/viscous_shock_tube/viscous_shock_tube.py: TENO5 with
the Roe average, central viscous terms with the constant viscosity mu = 1 (Re = 200, Pr = 0.73, Minf =
1), adiabatic walls on both x0 faces and at x1 = 0 (ReducedAccess closures), a symmetry face at the top
(central derivatives over its mirrored halos), RungeKuttaLS(3).

* FP64 GPU vs the reference's generated code (golden fixture ref_viscous_shock_tube: 48 x 24, 40 steps
  at dt = 1e-3) <= 1e-12.
* FP64 GPU vs the oracle for WENO5-JS and for Carpenter closures on the walls <= 1e-12; the
  right-hand side <= 1e-11.
* Graph replay and eager launches give bitwise equal states; mixed precision within 1e-5 (relative L2).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import viscous_shock_tube_plan
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu

INNER = (slice(None), slice(4, -4), slice(4, -4))


def golden():
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_viscous_shock_tube.npz"))
    return d["q0"], d["q"], tuple(int(x) for x in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def run_gpu(plan, q0, steps):
    s = Solver(plan)
    s.set_state64_padded(q0, 4)
    s.step(steps, plan.dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def rel_err_mom(a, b):
    """Max-normalised per variable, the momenta on the larger momentum's scale."""
    mom = max(float(np.abs(b[1]).max()), float(np.abs(b[2]).max()))
    return [float(np.abs(a[v] - b[v]).max() / (mom if v in (1, 2) else np.abs(b[v]).max())) for v in range(4)]


def test_viscous_shock_tube_fp64_matches_reference_golden():
    q0, q_ref, n, steps, params = golden()
    q = run_gpu(viscous_shock_tube_plan(*n, dt=params["dt"]), q0, steps)
    err = rel_err_mom(q, q_ref[INNER])
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("conv,closure", [("weno5js", "reduced_access"), ("teno5", "carpenter")])
def test_viscous_shock_tube_fp64_matches_oracle(conv, closure):
    q0, _, n, _, params = golden()
    plan = viscous_shock_tube_plan(*n, dt=params["dt"], conv=conv).replace(
        closure=((closure, closure), (closure, "none")))
    q = run_gpu(plan, q0, 30)
    q_or = O.run2d(plan, q0, 30)[INNER]
    assert max(rel_err_mom(q, q_or)) <= 1e-12, rel_err_mom(q, q_or)


def test_viscous_shock_tube_residual_graph_and_mixed():
    q0, q_ref, n, steps, params = golden()
    plan = viscous_shock_tube_plan(*n, dt=params["dt"])
    r_or = O.residual2d(plan, q_ref)
    s = Solver(plan)
    s.set_state64_padded(q_ref, 4)
    r = s.residual().cpu().numpy()
    s.close()
    err = [float(np.abs(r[v] - r_or[v]).max() / np.abs(r_or[v]).max()) for v in range(4)]
    assert max(err) <= 1e-11, err
    a = run_gpu(plan, q0, 6)
    b = run_gpu(plan.replace(use_graphs=False), q0, 6)
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), q0, steps)
    ref = q_ref[INNER]
    mom = float(np.linalg.norm(ref[1]))
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / (mom if v in (1, 2) else np.linalg.norm(ref[v]))) for v in range(4)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2


# ---- the laminar channel (apps/channel_flow/laminar_2D/laminar_channel.py): central skew-symmetric
# convective terms, Sutherland viscosity, periodic x0, isothermal walls on both x1 faces, forcing ----

def test_laminar_channel_fp64_matches_reference_golden_and_oracle():
    from opensbli_gb300.plan import laminar_channel_plan
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_laminar_channel.npz"))
    n = tuple(int(x) for x in d["n"])
    plan = laminar_channel_plan(*n, dt=json.loads(str(d["params"]))["dt"])
    q = run_gpu(plan, d["q0"], int(d["steps"]))
    assert max(rel_err_mom(q, d["q"][INNER])) <= 1e-12, rel_err_mom(q, d["q"][INNER])
    p2 = plan.replace(closure=(("none", "none"), ("reduced_access", "reduced_access")))
    assert max(rel_err_mom(run_gpu(p2, d["q0"], 20), O.run2d(p2, d["q0"], 20)[INNER])) <= 1e-12
    r_or = O.residual2d(plan, d["q"])
    s = Solver(plan)
    s.set_state64_padded(d["q"], 4)
    r = s.residual().cpu().numpy()
    s.close()
    mom = max(np.abs(r_or[1]).max(), np.abs(r_or[2]).max())
    assert max(float(np.abs(r[v] - r_or[v]).max() / (mom if v in (1, 2) else np.abs(r_or[v]).max())) for v in range(4)) <= 1e-11


def test_laminar_channel_graph_and_mixed():
    from opensbli_gb300.plan import laminar_channel_plan
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_laminar_channel.npz"))
    n = tuple(int(x) for x in d["n"])
    plan = laminar_channel_plan(*n, dt=json.loads(str(d["params"]))["dt"])
    assert np.array_equal(run_gpu(plan, d["q0"], 6), run_gpu(plan.replace(use_graphs=False), d["q0"], 6))
    qm = run_gpu(plan.replace(precision="mixed"), d["q0"], int(d["steps"]))
    ref = d["q"][INNER]
    mom = float(np.linalg.norm(ref[1]))
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / (mom if v in (1, 2) else np.linalg.norm(ref[v]))) for v in range(4)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2
