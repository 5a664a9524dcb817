"""GPU parity: libosbli_gb300 through its C ABI against the oracle and the reference's own output.

FP64 path: max-normalised error per conserved variable <= 1e-12 after the stated steps (the
bar the FP64 GPU path is held to against the reference's generated code).  Mixed path (FP32 state
and flux arithmetic, FP64 RK accumulator): relative L2 error vs the FP64 oracle <= 1e-5 after
a few steps on these small grids.
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as O
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver, OSBError
from helpers import load_golden, golden_plan, oracle_cfg, rel_err, rel_err_mom, rel_l2, WENOZ_TOL

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def run_gpu(plan, q0, steps, dt):
    s = Solver(plan)
    s.set_state64(q0)
    s.step(steps, dt)
    out = s.state64().cpu().numpy()
    s.close()
    return out


@pytest.mark.parametrize("case", ["tgv_central", "tgv_weno", "tgv_wenoz", "tgv_teno", "tgv_teno6", "tgsym_central"])
def test_gpu_fp64_matches_reference_golden(case):
    """The writer-lowered plan of the reference's own script reproduces the reference's output."""
    q_ref, n, steps, params = load_golden(case)
    plan = golden_plan(case, n=n).replace(Minf=params.get("Minf", 0.1))
    q0 = O.tgv_init(oracle_cfg(plan, dt=params["dt"]))
    q = run_gpu(plan, q0, steps, params["dt"])
    if plan.conv == "weno5z":  # the reference's own rounding noise floor (helpers.WENOZ_TOL)
        assert max(rel_err_mom(q, q_ref)) <= WENOZ_TOL
        return
    err = rel_err(q, q_ref)
    assert max(err) <= FP64_TOL, err


@pytest.mark.parametrize("conv,n,steps,dt,M", [
    ("central_skew", (24, 24, 24), 20, 5e-3, 0.1),
    ("central_skew", (40, 20, 16), 10, 5e-3, 0.1),
    ("weno5js", (20, 20, 20), 8, 2e-3, 1.25),
    ("weno5js", (70, 33, 18), 4, 2e-3, 1.25),
    ("weno5z", (20, 20, 20), 8, 2e-3, 1.25),
    ("weno5z", (33, 40, 17), 4, 2e-3, 1.25),
    ("teno5", (20, 20, 20), 8, 2e-3, 1.25),
    ("teno5", (33, 40, 17), 4, 2e-3, 1.25),
    ("teno6", (20, 20, 20), 8, 2e-3, 1.25),
    ("teno6", (33, 40, 17), 4, 2e-3, 1.25),
])
def test_gpu_fp64_matches_oracle(conv, n, steps, dt, M):
    plan = tgv_plan(n, conv=conv, Minf=M)
    cfg = oracle_cfg(plan, dt=dt)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, steps)
    q = run_gpu(plan, q0, steps, dt)
    if conv == "weno5z":
        assert max(rel_err_mom(q, q_or)) <= WENOZ_TOL
        return
    err = rel_err(q, q_or)
    assert max(err) <= FP64_TOL, err


@pytest.mark.parametrize("conv,M", [("central_skew", 0.1), ("weno5js", 1.25), ("teno5", 1.25), ("teno6", 1.25)])
def test_gpu_residual_matches_oracle(conv, M):
    plan = tgv_plan(24, conv=conv, Minf=M)
    cfg = oracle_cfg(plan)
    q0 = O.tgv_init(cfg)
    r_or = O.residual(cfg, q0)
    s = Solver(plan)
    s.set_state64(q0)
    r = s.residual().cpu().numpy()
    s.close()
    for v in range(5):
        scale = np.abs(r_or).max()
        assert np.abs(r[v] - r_or[v]).max() / scale <= FP64_TOL


@pytest.mark.parametrize("conv,M,tol", [("central_skew", 0.1, 2e-6), ("weno5js", 1.25, 2e-6), ("teno5", 1.25, 2e-6),
                                        ("teno6", 1.25, 2e-6)])
def test_gpu_mixed_close_to_fp64(conv, M, tol):
    plan = tgv_plan(32, conv=conv, Minf=M)
    cfg = oracle_cfg(plan, dt=2e-3)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 5)
    q = run_gpu(plan.replace(precision="mixed"), q0, 5, 2e-3)
    # rhou2 starts at zero and is still small after 5 steps: measure its error on the momentum
    # scale (the norm of rhou0) rather than on its own small norm
    l2 = rel_l2(q, q_or)
    l2[3] = float(np.linalg.norm(q[3] - q_or[3]) / np.linalg.norm(q_or[1]))
    assert max(l2) < tol, l2


def test_gpu_graph_and_eager_identical():
    q0 = O.tgv_init(oracle_cfg(tgv_plan(24, conv="weno5js", Minf=1.25)))
    a = run_gpu(tgv_plan(24, conv="weno5js", Minf=1.25, use_graphs=True), q0, 5, 2e-3)
    b = run_gpu(tgv_plan(24, conv="weno5js", Minf=1.25, use_graphs=False), q0, 5, 2e-3)
    assert np.array_equal(a, b)


def test_gpu_odd_even_step_counts_keep_state_in_bound_buffer():
    plan = tgv_plan(16)
    cfg = oracle_cfg(plan, dt=5e-3)
    q0 = O.tgv_init(cfg)
    s = Solver(plan)
    s.set_state64(q0)
    s.step(3, 5e-3)
    s.step(2, 5e-3)
    q = s.state64().cpu().numpy()
    # the bound arrays hold the same state as the FP64 register (FP64 mode)
    bound = np.stack([s.interior(v).cpu().numpy() for v in range(5)])
    s.close()
    assert np.array_equal(q, bound)
    assert max(rel_err(q, O.run(cfg, q0, 5))) <= FP64_TOL


def test_gpu_init_tgv_and_reductions():
    plan = tgv_plan(32)
    cfg = oracle_cfg(plan, dt=5e-3)
    q0 = O.tgv_init(cfg)
    s = Solver(plan)
    s.init_tgv()
    q = s.state64().cpu().numpy()
    assert max(rel_err(q, q0)) < 1e-15 * 10
    q_or, ke = O.run(cfg, q0, 4, with_ke=True)
    assert abs(s.reduce("ke") - ke[0]) / ke[0] < 1e-14
    s.step(4, 5e-3)
    assert abs(s.reduce("ke") - ke[4]) / ke[4] < 1e-12
    # enstrophy against a numpy evaluation of the same 4th-order central curl
    qs = s.state64().cpu().numpy()
    u = [qs[1 + c] / qs[0] for c in range(3)]
    d = plan.delta
    def d1(f, ax):  # arrays are [z][y][x]; axis 0 (x) is numpy axis 2
        a = 2 - ax
        return (np.roll(f, 2, a) / 12 - 2 * np.roll(f, 1, a) / 3 + 2 * np.roll(f, -1, a) / 3 - np.roll(f, -2, a) / 12) / d[ax]
    w0 = d1(u[2], 1) - d1(u[1], 2)
    w1 = d1(u[0], 2) - d1(u[2], 0)
    w2 = d1(u[1], 0) - d1(u[0], 1)
    ens = float(np.mean(0.5 * qs[0] * (w0 ** 2 + w1 ** 2 + w2 ** 2)))
    assert abs(s.reduce("enstrophy") - ens) / ens < 1e-12
    assert s.reduce("nancheck") == 0.0
    s.close()


def test_gpu_nancheck_flags_nonfinite_state():
    s = Solver(tgv_plan(16))
    s.init_tgv()
    torch.cuda.synchronize()
    s.interior(4)[3, 2, 1] = float("nan")
    with pytest.raises(OSBError, match="non-finite"):
        s.reduce("nancheck")
    s.close()


def test_gpu_plan_errors_surface_as_exceptions():
    with pytest.raises(OSBError):  # the adaptive cut-off needs TENO fluxes
        Solver(tgv_plan(32).replace(conv="weno5js", teno_adaptive=True))
    with pytest.raises(NotImplementedError):  # Sutherland viscosity is implemented on 2D blocks
        Solver(tgv_plan(32).replace(visc="sutherland"))
    s = Solver(tgv_plan(16))
    with pytest.raises(OSBError):
        s.step(1, -1.0)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_host_state_in_and_out_without_staging(precision):
    """set_state64 from a pinned host tensor (read by the kernels over the host link) and
    state64(out=pinned host tensor) give the same state as the device-array path; a pageable host
    pointer handed to the C entry point directly is refused, not read."""
    import ctypes
    plan = tgv_plan(20, conv="weno5js", Minf=1.25, precision=precision)
    q0 = O.tgv_init(oracle_cfg(plan, dt=2e-3))
    host = torch.from_numpy(q0).pin_memory()
    a = Solver(plan)
    a.set_state64(torch.from_numpy(q0).cuda())
    a.step(3, 2e-3)
    ref = a.state64().cpu()
    a.close()
    b = Solver(plan)
    b.set_state64(host)
    b.step(3, 2e-3)
    out = torch.empty_like(host).pin_memory()
    got = b.state64(out=out)
    assert got.data_ptr() == out.data_ptr() and torch.equal(out, ref)
    pageable = torch.from_numpy(q0.copy())
    rc = b.lib.osb_set_state64(b.ctx, 0, ctypes.c_void_p(pageable[0].data_ptr()))
    assert rc != 0
    b.close()
