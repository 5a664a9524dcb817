"""In-loop point monitors and the NaN check: the GB300 counterpart of SimulationMonitor
(core/diagnostics/simulation_monitors.py) and of the Condition the algorithm wraps it in
(code_generation/algorithm/algorithm.py:431-437).

The reference samples each monitored array at one grid point after the time step of iterations
iter = 0 and (iter+1) % print_frequency == 0, prints "Iteration, Time, <name>(i, j, k)..." once and then
one line per sample ("%d, %.<p>f, ..." with iter+1 and (iter+1)*dt), and with NaNcheck=True calls
ops_NaNcheck on the first monitored array, which aborts the run on a non-finite value.  Here the
samples come from osb_probe (FP64 state, one synchronising call per monitored iteration) and the
NaN check is osb_reduce(OSB_RED_NANCHECK) over the whole state, raising OSBError.
"""
import sys

from . import runtime

# names the probes understand: conserved variables by their OpenSBLI names, derived quantities
CONSERVED_3D = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]
CONSERVED_2D = ["rho", "rhou0", "rhou1", "rhoE"]
DERIVED = {"u0": 16, "u1": 17, "u2": 18, "p": 19, "T": 20}


def _name(a):
    """A DataSet (or its name) to the plain name: 'rho_B0' / DataSet rho -> 'rho'."""
    s = str(getattr(a, "base", a))
    return s.split("_B")[0] if "_B" in s else s


class SimulationMonitor:
    """Same arguments as the reference's SimulationMonitor(arrays, probe_locations, block, ...);
    `arrays` may be DataSets or names (conserved variables, or u0, u1, u2, p, T)."""

    def __init__(self, arrays, probe_locations, block=None, print_frequency=250, fp_precision=10, NaNcheck=True,
                 output_file=None):
        if len(arrays) != len(probe_locations):
            raise ValueError("The number of arrays must equal the number of probe locations.")
        self.names = [_name(a) for a in arrays]
        self.locations = [tuple(int(x) for x in (loc if isinstance(loc, (tuple, list)) else (loc,)))
                          for loc in probe_locations]
        self.frequency = int(print_frequency)
        self.fp_precision = int(fp_precision)
        self.NaNcheck = bool(NaNcheck)
        self.output_file = output_file
        self._out = None

    @classmethod
    def from_reference(cls, mon):
        """Build from the reference object an algorithm was given (TraditionalAlgorithmRK(...,
        simulation_monitor=...))."""
        return cls([m.flow_var for m in mon.monitors], [m.probe_loc for m in mon.monitors], None, mon.frequency,
                   mon.fp_precision, mon.NaNcheck, mon.output_file)

    def requests(self, ndim):
        cons = CONSERVED_3D if ndim == 3 else CONSERVED_2D
        req = []
        for name, loc in zip(self.names, self.locations):
            if name in cons:
                what = cons.index(name)
            elif name in DERIVED and not (ndim == 2 and name == "u2"):
                what = DERIVED[name]
            else:
                raise NotImplementedError("monitor of %r: only the conserved variables and u0..u2, p, T are held" % name)
            if len(loc) != ndim:
                raise ValueError("probe location %r does not have %d indices" % (loc, ndim))
            req.append((what,) + tuple(loc) + (0,) * (3 - ndim))
        return req

    def header(self):
        heads = ["Iteration", "Time"] + ["%s%s" % (n, str(loc)) for n, loc in zip(self.names, self.locations)]
        return ", ".join(heads)

    def line(self, iteration, time, values):
        fmt = "%%.%df" % self.fp_precision
        return ", ".join(["%d" % iteration, fmt % time] + [fmt % v for v in values])

    def _write(self, text):
        if self.output_file:
            if self._out is None:
                self._out = open(self.output_file, "a")
            self._out.write(text + "\n")
            self._out.flush()
        else:
            sys.stdout.write(text + "\n")

    def close(self):
        if self._out is not None:
            self._out.close()
            self._out = None

    def due(self, it):
        """Monitored after the step of iteration `it` (0-based), as the reference's Condition."""
        return it == 0 or (it + 1) % self.frequency == 0


def run(solver, niter, dt, monitor=None, t0_iteration=0):
    """Advance `niter` steps of `dt`, sampling and printing `monitor` (a SimulationMonitor) where the
    reference would.  Returns the list of (iteration, time, values) samples."""
    samples = []
    if monitor is None:
        solver.step(niter, dt)
        return samples
    req = monitor.requests(solver.plan.ndim)
    it = 0
    while it < niter:
        # steps up to and including the next monitored iteration
        nxt = it
        while nxt < niter - 1 and not monitor.due(t0_iteration + nxt):
            nxt += 1
        solver.step(nxt - it + 1, dt)
        it = nxt + 1
        g = t0_iteration + nxt
        if monitor.due(g):
            if monitor.NaNcheck:
                solver.reduce("nancheck")  # raises OSBError on a non-finite value
            vals = solver.probe(req)
            if g == 0:
                monitor._write(monitor.header())
            monitor._write(monitor.line(g + 1, (g + 1) * dt, vals))
            samples.append((g + 1, (g + 1) * dt, vals))
    return samples
