"""GPU: OPS-layout output and restart through Solver.write_ops_hdf5 / read_ops_hdf5."""
import numpy as np
import pytest

from oracle import oracle as O
from opensbli_gb300 import hdf5 as H
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver
from helpers import oracle_cfg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_from_output_continues_bitwise(precision, tmp_path):
    plan = tgv_plan(24, conv="weno5js", Minf=1.25, precision=precision)
    q0 = O.tgv_init(oracle_cfg(plan))
    dt = 2e-3
    a = Solver(plan)
    a.set_state64(q0)
    a.step(10, dt)
    q10 = a.state64().cpu().numpy()
    a.close()
    b = Solver(plan)
    b.set_state64(q0)
    b.step(4, dt)
    path = str(tmp_path / "opensbli_output_000004.h5")
    b.write_ops_hdf5(path)
    b.close()
    # the file holds the FP64 state with periodic 5-point halos
    arrays, halo, npts = H.read_ops_state(path, Solver(plan).state_names())
    assert halo == 5 and npts == (24, 24, 24) and arrays[0].shape == (34, 34, 34)
    assert np.array_equal(arrays[0][:5], arrays[0][24:29])
    c = Solver(plan)
    c.read_ops_hdf5(path)
    c.step(6, dt)
    assert np.array_equal(c.state64().cpu().numpy(), q10)
    c.close()


def test_output_with_extra_dats(tmp_path):
    plan = tgv_plan(16)
    s = Solver(plan)
    s.init_tgv()
    q = s.state64().cpu().numpy()
    x0 = np.broadcast_to(np.arange(16, dtype=np.float64) * plan.delta[0], (16, 16, 16)).copy()
    path = str(tmp_path / "o.h5")
    s.write_ops_hdf5(path, extra={"x0_B0": x0})
    s.close()
    root = H.read_file(path)["children"]["opensbliblock00"]["children"]
    assert sorted(root) == sorted(["rho_B0", "rhou0_B0", "rhou1_B0", "rhou2_B0", "rhoE_B0", "x0_B0"])
    assert np.array_equal(root["rhoE_B0"]["data"][5:-5, 5:-5, 5:-5], q[4])
    assert np.array_equal(root["x0_B0"]["data"][5:-5, 5:-5, 5:-5], x0)
