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


# Rounding sensitivity of the reference's own arithmetic on these fixtures (the oracle compiled with and
# without FMA contraction, max-normalised difference after the 20 steps): TENO5 and WENO5-JS 1e-15,
# TENO6 1.0e-12 (its sixth powers of (1 + tau/(eps + beta)) with eps = 1e-15 near the wall), WENO5-Z
# 3e-11 (eps = 1e-14).  Each bar sits a few times above that floor.
TOL_2D = {"katzer_teno": 1e-12, "katzer_weno": 1e-12, "katzer_teno6": 5e-12, "katzer_wenoz": 1e-9}


@pytest.mark.parametrize("case", sorted(TOL_2D))
def test_gpu_2d_fp64_matches_reference_golden(case):
    q0, x1, q_ref, n, steps, params = load_golden_2d(case)
    plan = golden_plan_2d(case, n=n).replace(dt=params["dt"])
    q = run_gpu_2d(plan, q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= TOL_2D[case], err


@pytest.mark.parametrize("case", ["katzer_weno", "katzer_wenoz", "katzer_teno6"])
def test_gpu_2d_schemes_fp64_match_oracle_and_mixed_close(case):
    """The other characteristic schemes on a wider block: FP64 against the oracle, mixed within 1e-5
    (relative L2) of FP64 after 10 steps."""
    q0, x1, _, n, _, params = load_golden_2d(case)
    q0w, x1w = widen_2d(q0, 96), widen_2d(x1[None], 96)[0]
    plan = golden_plan_2d(case, n=(96, n[1])).replace(dt=params["dt"])
    q_or = O.run2d(plan, q0w, 10)
    q = run_gpu_2d(plan, q0w, x1w, 10, params["dt"])
    ref = q_or[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= TOL_2D[case], err
    qm = run_gpu_2d(plan.replace(precision="mixed"), q0w, x1w, 10, params["dt"])
    l2 = [float(np.linalg.norm(qm[v] - q[v]) / np.linalg.norm(q[v])) for v in range(4)]
    assert max(l2) <= 1e-5, l2


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


# ---- the published Katzer script: TENO cut-off adapted per interface by the Ducros sensor ----

def test_gpu_2d_adaptive_fp64_matches_reference_golden():
    q0, x1, q_ref, n, steps, params = load_golden_2d("katzer_adaptive")
    plan = golden_plan_2d("katzer_adaptive", n=n).replace(dt=params["dt"])
    assert plan.teno_adaptive
    q = run_gpu_2d(plan, q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-12, err


def perturbed_state(n0, amp=0.03, seed=3):
    """The Katzer initial state widened to n0 columns with seeded noise on both momenta: the sensor
    then takes all five cut-off levels 1e-10 .. 1e-6 somewhere (the laminar state alone keeps
    C_T = 1e-10 almost everywhere)."""
    q0, x1, _, n, _, _ = load_golden_2d("katzer_adaptive")
    q, x1w = widen_2d(q0, n0), widen_2d(x1[None], n0)[0]
    rng = np.random.default_rng(seed)
    q[1] *= 1 + amp * rng.standard_normal(q[1].shape)
    q[2] += amp * rng.standard_normal(q[2].shape)
    return q, x1w, n


@pytest.mark.parametrize("n0,steps,perturb", [(130, 20, False), (96, 10, True)])
def test_gpu_2d_adaptive_fp64_matches_oracle(n0, steps, perturb):
    dt = 0.01
    if perturb:
        q0w, x1w, n = perturbed_state(n0)
    else:
        q0, x1, _, n, _, _ = load_golden_2d("katzer_adaptive")
        q0w, x1w = widen_2d(q0, n0), widen_2d(x1[None], n0)[0]
    plan = golden_plan_2d("katzer_adaptive", n=(n0, n[1])).replace(dt=dt)
    q_or = O.run2d(plan, q0w, steps)
    q = run_gpu_2d(plan, q0w, x1w, steps, dt)
    ref = q_or[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-11, err


def test_gpu_2d_adaptive_cutoff_field_matches_oracle():
    """The per-point cut-off (the reference's TENO_B0 field), bit for bit, on a state where the
    sensor takes every level."""
    q, x1w, n = perturbed_state(96)
    plan = golden_plan_2d("katzer_adaptive", n=(96, n[1])).replace(dt=0.01)
    ct_or = O.cutoff2d(plan, q)
    s = Solver(plan)
    s.set_coordinate(x1w, 4)
    s.set_state64_padded(q, 4)
    ct = s.teno_cutoff().cpu().numpy()
    s.close()
    assert len(np.unique(ct_or)) == 5
    assert np.array_equal(ct, ct_or), int((ct != ct_or).sum())


def test_gpu_2d_adaptive_mixed_close_to_fp64():
    q0, x1, q_ref, n, steps, params = load_golden_2d("katzer_adaptive")
    plan = golden_plan_2d("katzer_adaptive", n=n).replace(dt=params["dt"])
    qm = run_gpu_2d(plan.replace(precision="mixed"), q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / np.linalg.norm(ref[v])) for v in range(4)]
    assert max(l2) < 1e-5, l2


def test_gpu_2d_adaptive_graph_and_eager_identical():
    q0, x1, _, n, _, params = load_golden_2d("katzer_adaptive")
    plan = golden_plan_2d("katzer_adaptive", n=n).replace(dt=params["dt"])
    a = run_gpu_2d(plan.replace(use_graphs=True), q0, x1, 4, params["dt"])
    b = run_gpu_2d(plan.replace(use_graphs=False), q0, x1, 4, params["dt"])
    assert np.array_equal(a, b)


def test_gpu_2d_cutoff_needs_an_adaptive_plan():
    q0, x1, _, n, _, params = load_golden_2d("katzer_teno")
    plan = golden_plan_2d("katzer_teno", n=n).replace(dt=params["dt"])
    s = Solver(plan)
    s.set_coordinate(x1, 4)
    s.set_state64_padded(q0, 4)
    with pytest.raises(Exception):
        s.teno_cutoff()
    s.close()


# ---- Carpenter closures (the reference's default; here on the outlet and the wall) ----

def test_gpu_2d_carpenter_fp64_matches_reference_golden():
    q0, x1, q_ref, n, steps, params = load_golden_2d("katzer_carpenter")
    plan = golden_plan_2d("katzer_carpenter", n=n).replace(dt=params["dt"])
    assert plan.closure == (("reduced_access", "carpenter"), ("carpenter", "reduced_access"))
    q = run_gpu_2d(plan, q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-12, err


@pytest.mark.parametrize("closure", [(("carpenter", "reduced_access"), ("reduced_access", "carpenter")),
                                     (("carpenter", "carpenter"), ("carpenter", "carpenter"))])
def test_gpu_2d_carpenter_fp64_matches_oracle(closure):
    """Every face combination the golden case does not hold, on a wider grid and a perturbed state."""
    q0, x1, _, n, _, params = load_golden_2d("katzer_carpenter")
    q0w, x1w = widen_2d(q0, 96), widen_2d(x1[None], 96)[0]
    rng = np.random.default_rng(3)
    q0w = q0w * (1.0 + 1e-3 * rng.standard_normal(q0w.shape))
    plan = golden_plan_2d("katzer_carpenter", n=(96, n[1])).replace(dt=params["dt"], closure=closure)
    q_or = O.run2d(plan, q0w, 10)
    q = run_gpu_2d(plan, q0w, x1w, 10, params["dt"])
    ref = q_or[:, 4:-4, 4:-4]
    err = [float(np.abs(q[v] - ref[v]).max() / np.abs(ref[v]).max()) for v in range(4)]
    assert max(err) <= 1e-12, err


def test_gpu_2d_carpenter_mixed_close_to_fp64():
    q0, x1, q_ref, n, steps, params = load_golden_2d("katzer_carpenter")
    plan = golden_plan_2d("katzer_carpenter", n=n).replace(dt=params["dt"], precision="mixed")
    qm = run_gpu_2d(plan, q0, x1, steps, params["dt"])
    ref = q_ref[:, 4:-4, 4:-4]
    l2 = [float(np.linalg.norm(qm[v] - ref[v]) / np.linalg.norm(ref[v])) for v in range(4)]
    assert max(l2) < 1e-5, l2
