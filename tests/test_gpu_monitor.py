"""GPU: point probes (osb_probe) and the monitored time loop against the FP64 state and the oracle."""
import io
import contextlib

import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300 import monitor as M
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver, OSBError
from helpers import oracle_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_monitored_run_matches_oracle(precision, tmp_path):
    plan = tgv_plan((16, 14, 12), precision=precision)
    dt = 5e-3
    cfg = oracle_cfg(plan, dt=dt)
    q0 = O.tgv_init(cfg)
    s = Solver(plan)
    s.set_state64(q0)
    mon = M.SimulationMonitor(["rho", "rhou1", "p", "T"], [(3, 4, 5), (1, 2, 3), (15, 13, 11), (0, 0, 0)],
                              print_frequency=4, fp_precision=12, output_file=str(tmp_path / "mon.log"))
    samples = M.run(s, 10, dt, mon)
    mon.close()
    s.close()
    assert [it for it, _, _ in samples] == [1, 4, 8]
    lines = open(tmp_path / "mon.log").read().splitlines()
    assert lines[0] == "Iteration, Time, rho(3, 4, 5), rhou1(1, 2, 3), p(15, 13, 11), T(0, 0, 0)"
    assert len(lines) == 4 and lines[2].startswith("4, 0.020000000000")
    g, gm2 = plan.gama - 1.0, plan.gama * plan.Minf ** 2
    tol = 1e-12 if precision == "fp64" else 1e-5
    for it, _, vals in samples:
        q = O.run(cfg, q0, it)
        rho, ru1 = q[0][5, 4, 3], q[2][3, 2, 1]
        qq = q[:, 11, 13, 15]
        p = g * (qq[4] - 0.5 * (qq[1] ** 2 + qq[2] ** 2 + qq[3] ** 2) / qq[0])
        q0p = q[:, 0, 0, 0]
        p0 = g * (q0p[4] - 0.5 * (q0p[1] ** 2 + q0p[2] ** 2 + q0p[3] ** 2) / q0p[0])
        ref = [rho, ru1, p, gm2 * p0 / q0p[0]]
        for a, b in zip(vals, ref):
            assert abs(a - b) <= tol * max(1.0, abs(b))


def test_probe_rejects_out_of_range():
    s = Solver(tgv_plan(12))
    s.init_tgv()
    with pytest.raises(OSBError):
        s.probe([(0, 12, 0, 0)])
    with pytest.raises(OSBError):
        s.probe([(7, 0, 0, 0)])
    assert s.probe([(0, 1, 1, 1)])[0] > 0
    s.close()
