"""GPU parity of the 2D curvilinear wall-bounded path (TENO5, metrics, Sutherland viscosity,
isothermal wall, inlet/outlet/Dirichlet faces, LS-RK3) against the reference's own output and the
oracle.  FP64: max-normalised interior error <= 1e-12; mixed: relative L2 <= 1e-5 after 20 steps."""
import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.runtime import Solver
from helpers import load_golden_2d, golden_plan_2d, widen_2d, rel_err_2d

pytestmark = pytest.mark.gpu


def run_gpu_2d(plan, q0_pad, x1_pad, steps, dt):
    s = Solver(plan)
    s.set_coordinate(x1_pad, 4)
    s.set_state64_padded(q0_pad, 4)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def test_gpu_2d_fp64_matches_reference_golden():
    q0, x1, q_ref, n, steps, params = load_golden_2d()
    plan = golden_plan_2d(n=n).replace(dt=params["dt"])
    q = run_gpu_2d(plan, q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("n0,steps", [(70, 10), (130, 5)])
def test_gpu_2d_fp64_matches_oracle_wider_grids(n0, steps):
    q0, x1, _, n, _, params = load_golden_2d()
    q0w, x1w = widen_2d(q0, n0), widen_2d(x1[None], n0)[0]
    plan = golden_plan_2d(n=(n0, n[1])).replace(dt=params["dt"])
    q_or = O.run2d(plan, q0w, steps)
    q = run_gpu_2d(plan, q0w, x1w, steps, params["dt"])
    ref = q_or[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-12, err


def test_gpu_2d_mixed_close_to_fp64():
    q0, x1, q_ref, n, steps, params = load_golden_2d()
    plan = golden_plan_2d(n=n).replace(dt=params["dt"])
    qm = run_gpu_2d(plan.replace(precision="mixed"), q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / np.linalg.norm(ref[v])) for v in range(4)]
    assert max(l2) < 1e-5, l2


def test_gpu_2d_graph_and_eager_identical():
    q0, x1, _, n, _, params = load_golden_2d()
    plan = golden_plan_2d(n=n).replace(dt=params["dt"])
    a = run_gpu_2d(plan.replace(use_graphs=True), q0, x1, 4, params["dt"])
    b = run_gpu_2d(plan.replace(use_graphs=False), q0, x1, 4, params["dt"])
    assert np.array_equal(a, b)


def test_gpu_2d_reductions():
    q0, x1, _, n, _, params = load_golden_2d()
    plan = golden_plan_2d(n=n).replace(dt=params["dt"])
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0, 4)
    q = q0[:, 4:-4, 4:-4]
    ke = float(np.mean(0.5 * (q[1] ** 2 + q[2] ** 2) / q[0]))
    assert abs(s.reduce("ke") - ke) / ke < 1e-13
    assert s.reduce("nancheck") == 0.0
    with pytest.raises(NotImplementedError):
        s.reduce("enstrophy")
    s.close()
