"""GPU: every launch shape of the WENO5-JS flux kernels gives the oracle's residual, and the autotuner
keeps a valid shape.

Shapes: the tiled kernel (all directions) and the line-marching kernel (y and z) with 4 or 8 lines
per block and segment lengths that do and do not divide the line (ragged last segment, a segment
longer than the line).  FP64: max-normalised residual error <= 1e-11 against the oracle; states after
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
    for d in (1, 2):
        s.set_weno_shape(d, kind, seg)
        assert s.weno_shape(d) == (kind, seg)
    r = s.residual().double().cpu().numpy()
    s.close()
    return r


@pytest.mark.parametrize("n", [(24, 24, 24), (40, 37, 29)])
@pytest.mark.parametrize("kind,seg", SHAPES)
def test_weno_shapes_fp64_match_oracle(n, kind, seg):
    plan = tgv_plan(n, conv="weno5js", Minf=1.25)
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
    for r in rs[1:]:
        assert np.abs(r - rs[0]).max() / scale <= 1e-5


def test_weno_shape_steps_match_oracle():
    """A few RK3 steps with a line-marching shape through the captured-graph path."""
    plan = tgv_plan((33, 30, 27), conv="weno5js", Minf=1.25)
    cfg = oracle_cfg(plan, dt=2e-3)
    q0 = O.tgv_init(cfg)
    q_or = O.run(cfg, q0, 4)
    s = Solver(plan)
    s.set_state64(q0)
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
    assert set(best) == {0, 1, 2}
    for d, (kind, seg, ms) in best.items():
        assert kind in ("tile", "march4", "march8") and 4 <= seg <= 4096 and ms > 0
    assert best[0][0] == "tile"
    r1 = s.residual().double().cpu().numpy()
    s.close()
    assert np.abs(r1 - r0).max() / np.abs(r0).max() <= 1e-5


def test_shape_rejections():
    s = Solver(tgv_plan(16, conv="weno5js", Minf=1.25))
    with pytest.raises(NotImplementedError):
        s.set_weno_shape(0, "march4", 32)
    with pytest.raises(OSBError):
        s.set_weno_shape(1, "march4", 2)
    with pytest.raises(OSBError):
        s.set_weno_shape(3, "tile", 32)
    s.close()


def test_autotune_noop_without_weno():
    s = Solver(tgv_plan(16))
    s.init_tgv()
    assert s.autotune(reps=1) == {}
    s.close()
