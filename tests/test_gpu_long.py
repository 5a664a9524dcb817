"""GPU: long runs of the plain FP64 path against the reference's own generated code (built from
oracle/_ref with the OPS-API stand-in and run on the host cores), at the configurations' stated step
counts where the host can afford them, and the mixed path's error against the FP64 path.

* Taylor-Green 64^3, central skew-symmetric + viscous, Minf 0.1, dt 5e-3, 200 RK3 steps: FP64 GPU vs
  reference <= 1e-12 (max-normalised, per conserved variable).
* Taylor-Green 64^3, WENO5-JS + viscous, Minf 1.25, dt from CFL 0.5, 200 steps: FP64 GPU vs reference.
* Katzer 2D SBLI 512x256, TENO5 + metrics, 500 of the 5000 steps (the reference takes ~15 s per 500 on
  16 cores): FP64 GPU vs reference, from the reference's own initial state.
Each also reports (in the assertion message) the mixed path's relative L2 error against FP64.
"""
import os
import tempfile

import numpy as np
import pytest

from oracle import refrun
from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt
from opensbli_gb300.runtime import Solver
from helpers import golden_plan_2d, rel_err, rel_err_2d

pytestmark = pytest.mark.gpu
VARS = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]
VARS_2D = ["rho", "rhou0", "rhou1", "rhoE"]
THREADS = min(16, os.cpu_count() or 1)


def gpu_run(plan, steps, dt, q0=None):
    s = Solver(plan)
    if q0 is None:
        s.init_tgv()
    else:
        s.set_state64(q0)
    s.step(steps, dt)
    q = s.state64().cpu().numpy()
    s.close()
    return q


def rel_l2(a, b):
    return [float(np.linalg.norm(a[v] - b[v]) / np.linalg.norm(b[v])) for v in range(b.shape[0])]


@pytest.mark.parametrize("case,conv,M", [("tgv_central", "central_skew", 0.1), ("tgv_weno", "weno5js", 1.25)])
def test_fp64_matches_reference_200_steps(case, conv, M):
    if not refrun.available(case):
        pytest.skip("generated reference sources for %s not present" % case)
    n, steps = 64, 200
    plan = tgv_plan(n, conv=conv, Minf=M)
    dt = 5e-3 if conv == "central_skew" else tgv_cfl_dt(plan)
    fields, _ = refrun.run(case, dict(block0np0=n, block0np1=n, block0np2=n, niter=steps, dt=dt, Minf=M), VARS,
                           threads=THREADS)
    q_ref = np.stack([fields[v] for v in VARS])
    q64 = gpu_run(plan, steps, dt)
    qm = gpu_run(plan.replace(precision="mixed"), steps, dt)
    err = rel_err(q64, q_ref)
    assert max(err) <= 1e-12, (err, "mixed L2 vs fp64", rel_l2(qm, q64))


def test_katzer_fp64_matches_reference_500_steps():
    case = "katzer_teno"
    if not refrun.available(case):
        pytest.skip("generated reference sources for %s not present" % case)
    (n0, n1), steps, dt = (512, 256), 500, 0.04
    base = dict(block0np0=n0, block0np1=n1, dt=dt)
    d0 = tempfile.mkdtemp(prefix="osb_k0_")
    refrun.run(case, dict(base, niter=0), VARS_2D + ["x1"], threads=THREADS, outdir=d0)
    pad = lambda d, v: refrun.load_dump(os.path.join(d, "opensbli_output.%s_B0.bin" % v), interior=False)[1:-1, 1:-1]
    q0 = np.stack([pad(d0, v) for v in VARS_2D])
    x1 = pad(d0, "x1")
    d1 = tempfile.mkdtemp(prefix="osb_k1_")
    refrun.run(case, dict(base, niter=steps), VARS_2D, threads=THREADS, outdir=d1)
    q_ref = np.stack([pad(d1, v) for v in VARS_2D])
    out = {}
    for prec in ("fp64", "mixed"):
        plan = golden_plan_2d(n=(n0, n1)).replace(dt=dt, precision=prec)
        s = Solver(plan)
        s.set_coordinate(x1, 4)
        s.set_state64_padded(q0, 4)
        s.step(steps, dt)
        out[prec] = s.state64().cpu().numpy()
        s.close()
    h = 4
    ref_int = q_ref[:, h:-h, h:-h]
    err = rel_err(out["fp64"], ref_int)
    assert max(err) <= 1e-12, (err, "mixed L2 vs fp64", rel_l2(out["mixed"], out["fp64"]))


def test_mixed_weno_error_budget_128_500_steps():
    """Mixed path (FP32 state and arithmetic, FP64 RK register) against the FP64 path: Taylor-Green
    128^3, WENO5-JS + viscous, Minf 1.25, CFL 0.5, 500 steps (the same physical time as 1000 steps
    at 256^3).  Measured 3.6e-8 .. 1.3e-7 relative L2; the bound leaves a factor of two.  Larger
    errors here mean FP32 rounding noise or a one-sided bias came back: the primitives rounded
    once, the difference-form characteristic flux, the differenced central stencils and the hi/lo
    FP32 constants are what keep it down."""
    plan = tgv_plan(128, conv="weno5js", Minf=1.25)
    dt = tgv_cfl_dt(plan)
    q64 = gpu_run(plan, 500, dt)
    qm = gpu_run(plan.replace(precision="mixed"), 500, dt)
    l2 = rel_l2(qm, q64)
    assert np.isfinite(qm).all() and max(l2) <= 3e-7, l2


def test_mixed_weno_256_1000_steps_within_1e6():
    """The headline accuracy bar: Taylor-Green 256^3, WENO5-JS + viscous, Minf 1.25, CFL 0.5, the full
    1000 RK3 steps; the mixed path's relative L2 error against the FP64 path must stay within 1e-6 on
    every conserved variable (Linf is reported in the message).  The FP64 run takes about five and a
    half minutes on one GB300."""
    plan = tgv_plan(256, conv="weno5js", Minf=1.25)
    dt = tgv_cfl_dt(plan)
    q64 = gpu_run(plan, 1000, dt)
    qm = gpu_run(plan.replace(precision="mixed"), 1000, dt)
    l2 = rel_l2(qm, q64)
    linf = [float(np.abs(qm[v] - q64[v]).max() / np.abs(q64[v]).max()) for v in range(5)]
    assert np.isfinite(qm).all() and np.isfinite(q64).all()
    assert max(l2) <= 1e-6, ("L2", dict(zip(VARS, l2)), "Linf", dict(zip(VARS, linf)))
