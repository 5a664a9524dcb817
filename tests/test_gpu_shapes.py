"""GPU: every launch shape of the WENO5-JS flux kernels gives the oracle's residual, and the autotuner
keeps a valid shape.

Shapes: the tiled kernel and the line-marching kernels (x: warps over 32 y-lines with a per-warp
shared-memory transpose; y, z: one line per thread) with 4 or 8 warps per block and segment lengths
that do and do not divide the line (ragged last segment, a segment longer than the line).  FP64: max-normalised residual error <= 1e-11 against the oracle; states after
RK3 steps <= 1e-12.  Mixed: the shapes agree with one another to FP32 rounding.

Why 1e-11 for a single residual: the reference evaluates the WENO5-JS smoothness indicators in an
expanded product form (weno.py) whose terms are O(f^2) and cancel to O(beta); with eps = 1e-6 the
weights amplify that rounding by ~1/eps where beta << eps.  The oracle (the reference's arithmetic)
compiled with and without FMA contraction differs from itself by 2.8e-12 at 40x37x29 and 7.8e-12 at
70x33x18 in this norm, the same size as its difference from these kernels (which use the
sum-of-squares form).  After RK3 steps the residual is scaled by dt and the bar is 1e-12 again.
"""
import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver, OSBError
from helpers import oracle_cfg, rel_err

pytestmark = pytest.mark.gpu

SHAPES = [("tile", 32), ("march4", 16), ("march4", 7), ("march8", 32), ("march8", 64), ("march8", 500)]


def residual_with(plan, q0, kind, seg):
    s = Solver(plan)
    s.set_state64(q0)
    for d in (0, 1, 2):
        s.set_weno_shape(d, kind, seg)
        assert s.weno_shape(d) == (kind, seg)
    r = s.residual().double().cpu().numpy()
    s.close()
    return r


@pytest.mark.parametrize("conv", ["weno5js", "teno5", "teno6"])
@pytest.mark.parametrize("n", [(24, 24, 24), (40, 37, 29)])
@pytest.mark.parametrize("kind,seg", SHAPES)
def test_weno_shapes_fp64_match_oracle(n, kind, seg, conv):
    plan = tgv_plan(n, conv=conv, Minf=1.25)
    cfg = oracle_cfg(plan)
    q0 = O.tgv_init(cfg)
    r_or = O.residual(cfg, q0)
    r = residual_with(plan, q0, kind, seg)
    scale = np.abs(r_or).max()
    assert np.abs(r - r_or).max() / scale <= 1e-11


def test_weno_shapes_mixed_agree():
    plan = tgv_plan((48, 40, 36), conv="weno5js", Minf=1.25, precision="mixed")
    q0 = O.tgv_init(oracle_cfg(plan))
    rs = [residual_with(plan, q0, k, sg) for k, sg in SHAPES]
    scale = np.abs(rs[0]).max()
    # each kernel shape rounds its FP32 flux arithmetic in its own order; the flux difference
    # divided by delta (~0.13 here) turns O(1e-7) flux rounding into up to ~1e-5 of max |R|
    for r in rs[1:]:
        assert np.abs(r - rs[0]).max() / scale <= 5e-5


def test_weno_shape_steps_match_oracle():
    """A few RK3 steps with a line-marching shape through the captured-graph path."""
    plan = tgv_plan((33, 30, 27), conv="weno5js", Minf=1.25)
    cfg = oracle_cfg(plan, dt=2e-3)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 4)
    s = Solver(plan)
    s.set_state64(q0)
    s.set_weno_shape(0, "march4", 20)
    s.set_weno_shape(1, "march8", 16)
    s.set_weno_shape(2, "march4", 12)
    s.step(4, 2e-3)
    q = s.state64().cpu().numpy()
    s.close()
    assert max(rel_err(q, q_or)) <= 1e-12


def test_autotune_keeps_valid_shape_and_results():
    plan = tgv_plan(48, conv="weno5js", Minf=1.25, precision="mixed")
    q0 = O.tgv_init(oracle_cfg(plan))
    s = Solver(plan)
    s.set_state64(q0)
    r0 = s.residual().double().cpu().numpy()
    best = s.autotune(reps=2)
    assert set(best) == {"weno_x", "weno_y", "weno_z", "central"}
    for name in ("weno_x", "weno_y", "weno_z"):
        kind, seg, ms = best[name]
        assert kind in ("tile", "march4", "march8") and 4 <= seg <= 4096 and ms > 0
    assert best["central"][0] in (8, 16) and best["central"][1] > 0
    # the state is untouched: the residual agrees up to the FP32 rounding of the chosen shapes
    r1 = s.residual().double().cpu().numpy()
    s.close()
    assert np.abs(r1 - r0).max() / np.abs(r0).max() <= 5e-5


@pytest.mark.parametrize("conv,M", [("central_skew", 0.1), ("weno5js", 1.25)])
def test_autotune_leaves_state_alone(conv, M):
    plan = tgv_plan((40, 36, 32), conv=conv, Minf=M)
    cfg = oracle_cfg(plan, dt=2e-3)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 3)
    s = Solver(plan)
    s.set_state64(q0)
    s.step(1, 2e-3)
    s.autotune(reps=1)
    s.step(2, 2e-3)
    q = s.state64().cpu().numpy()
    s.close()
    assert max(rel_err(q, q_or)) <= 1e-12


@pytest.mark.parametrize("ty", [8, 16])
@pytest.mark.parametrize("conv,M", [("central_skew", 0.1), ("weno5js", 1.25)])
def test_central_shapes_match_oracle(ty, conv, M):
    plan = tgv_plan((37, 41, 30), conv=conv, Minf=M)
    cfg = oracle_cfg(plan, dt=2e-3)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 3)
    s = Solver(plan)
    s.set_state64(q0)
    s.set_central_shape(ty)
    assert s.central_shape() == ty
    s.step(3, 2e-3)
    q = s.state64().cpu().numpy()
    s.close()
    assert max(rel_err(q, q_or)) <= 1e-12


def test_shape_rejections():
    s = Solver(tgv_plan(16, conv="weno5js", Minf=1.25))
    with pytest.raises(OSBError):  # unknown kind code through the C ABI
        s._check(s.lib.osb_set_weno_shape(s.ctx, 0, 7, 32))
    with pytest.raises(OSBError):
        s.set_weno_shape(1, "march4", 2)
    with pytest.raises(OSBError):
        s.set_weno_shape(3, "tile", 32)
    with pytest.raises(OSBError):
        s.set_central_shape(12)
    s.close()


def test_autotune_central_only_plan():
    s = Solver(tgv_plan(16))
    s.init_tgv()
    best = s.autotune(reps=1)
    assert set(best) == {"central"} and best["central"][0] in (8, 16)
    s.close()
