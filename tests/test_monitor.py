"""Point monitors (opensbli_gb300/monitor.py) on CPU: the reference's sampling schedule (iteration 0
and every print_frequency-th, core/diagnostics/simulation_monitors.py with algorithm.py:431-437), its
header and line format, and construction from a reference-shaped SimulationMonitor object."""
import types

import pytest

from opensbli_gb300.monitor import SimulationMonitor


def test_schedule_header_and_format():
    m = SimulationMonitor(["rho", "p"], [(3, 4, 5), (1, 2, 3)], print_frequency=4, fp_precision=6)
    assert [it for it in range(12) if m.due(it)] == [0, 3, 7, 11]
    assert m.header() == "Iteration, Time, rho(3, 4, 5), p(1, 2, 3)"
    assert m.line(4, 0.02, [1.0, 71.4285714]) == "4, 0.020000, 1.000000, 71.428571"
    assert m.requests(3) == [(0, 3, 4, 5), (19, 1, 2, 3)]


def test_requests_and_errors():
    m = SimulationMonitor(["rhoE", "u2", "T"], [(0, 0, 0), (1, 1, 1), (2, 2, 2)])
    assert m.requests(3) == [(4, 0, 0, 0), (18, 1, 1, 1), (20, 2, 2, 2)]
    with pytest.raises(NotImplementedError):
        SimulationMonitor(["vorticity"], [(0, 0, 0)]).requests(3)
    with pytest.raises(ValueError):
        SimulationMonitor(["rho"], [(0, 0)]).requests(3)
    with pytest.raises(ValueError):
        SimulationMonitor(["rho", "p"], [(0, 0, 0)])
    assert SimulationMonitor(["rhoE", "u1"], [(5, 6), (7, 8)]).requests(2) == [(3, 5, 6, 0), (17, 7, 8, 0)]


def test_from_reference_shaped_object():
    mons = [types.SimpleNamespace(flow_var="rho_B0", probe_loc=(1, 2, 3)),
            types.SimpleNamespace(flow_var="rhou0_B0", probe_loc=(4, 5, 6))]
    ref = types.SimpleNamespace(monitors=mons, frequency=50, fp_precision=8, NaNcheck=False, output_file=None)
    m = SimulationMonitor.from_reference(ref)
    assert m.names == ["rho", "rhou0"] and m.locations == [(1, 2, 3), (4, 5, 6)]
    assert m.frequency == 50 and m.fp_precision == 8 and not m.NaNcheck
