"""Shared helpers for the tests: golden fixtures and oracle configurations."""
import json
import math
import os

import numpy as np

from oracle import oracle as O
from opensbli_gb300.plan import Plan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
VARS = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]


def load_golden(case):
    d = np.load(os.path.join(GOLDEN, "ref_%s.npz" % case))
    return d["q"], int(d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def golden_plan(case, n=None, **kw):
    with open(os.path.join(GOLDEN, "plan_%s.json" % case)) as f:
        p = Plan.from_json(f.read())
    if n is not None:
        if p.bc[0][0] == "symmetry":
            delta = (math.pi / (n - 1),) * 3
        else:
            delta = (2 * math.pi / n,) * 3
        p = p.replace(n=(n, n, n), delta=delta)
    return p.replace(**kw) if kw else p


def oracle_cfg(plan, dt=None):
    bc = [[plan.bc[d][s] for s in range(2)] for d in range(3)]
    return O.make_cfg(plan.n, plan.delta, gama=plan.gama, Minf=plan.Minf, Re=plan.Re, Pr=plan.Pr, conv=plan.conv,
                      visc=plan.visc, rk="rk3", bc=bc, dt=dt if dt is not None else (plan.dt or 1e-3),
                      filter=plan.filter, filter_control=plan.filter_control, teno_ct=plan.teno_ct,
                      teno_eps=plan.teno_eps, teno_adaptive=plan.teno_adaptive, teno_a1=plan.teno_a1,
                      teno_a2=plan.teno_a2, sensor_eps=plan.sensor_eps)


def rel_err(a, b):
    """max |a-b| / max |b| per variable."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = []
    for v in range(b.shape[0]):
        s = np.abs(b[v]).max()
        out.append(float(np.abs(a[v] - b[v]).max() / (s if s > 0 else 1.0)))
    return out


def rel_err_mom(a, b):
    """max |a-b| per variable, normalised by max |b| of the variable, except that the three momentum
    components share the largest momentum scale (a component that starts at zero, like rhou2 of the
    Taylor-Green vortex, is measured on the momentum scale rather than on its own small one)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    mom = max(float(np.abs(b[v]).max()) for v in (1, 2, 3))
    out = []
    for v in range(b.shape[0]):
        s = mom if v in (1, 2, 3) else float(np.abs(b[v]).max())
        out.append(float(np.abs(a[v] - b[v]).max() / (s if s > 0 else 1.0)))
    return out


# WENO5-Z with the reference's eps = 1e-14 amplifies rounding where a characteristic field is nearly
# flat (beta ~ rounding noise): the oracle compiled with and without FMA contraction differs from
# itself by 9e-9 (rho) .. 2e-8 (momentum scale) after one step at 16^3 and by 4e-8 .. 6e-8 after 10, as
# much as from the reference.  Parity for WENO5-Z is held at this bar (momentum-scale normalisation).
WENOZ_TOL = 2e-6


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return [float(np.linalg.norm(a[v] - b[v]) / max(np.linalg.norm(b[v]), 1e-300)) for v in range(b.shape[0])]


def load_golden_2d(case="katzer_teno"):
    d = np.load(os.path.join(GOLDEN, "ref_%s.npz" % case))
    return d["q0"], d["x1"], d["q"], tuple(int(v) for v in d["n"]), int(d["steps"]), json.loads(str(d["params"]))


def golden_plan_2d(case="katzer_teno", n=None, **kw):
    with open(os.path.join(GOLDEN, "plan_%s.json" % case)) as f:
        p = Plan.from_json(f.read())
    if n is not None:
        n0, n1 = n
        p = p.replace(n=(n0, n1, 1), delta=(400.0 / (n0 - 1), 115.0 / (n1 - 1), 1.0))
    return p.replace(**kw) if kw else p


def widen_2d(q_pad, n0_new):
    """A padded 2D state whose rows depend on x1 only, widened to n0_new interior columns by repeating
    its first interior column (the Katzer initial state is independent of x0)."""
    h = 4
    col = q_pad[..., :, h:h + 1]
    return np.repeat(col, n0_new + 2 * h, axis=-1)


def rel_err_2d(a, b, h=4):
    """max-normalised error over the interior of padded 2D states."""
    sl = (slice(h, -h), slice(h, -h))
    return [float(np.abs(a[v][sl] - b[v][sl]).max() / np.abs(b[v][sl]).max()) for v in range(b.shape[0])]
