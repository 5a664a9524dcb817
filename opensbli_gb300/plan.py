"""Plan: everything the GB300 kernels need to know about one block's time loop.

A Plan is what GB300Writer lowers an OpenSBLI algorithm to (the analogue of the constants,
datasets, kernel list and RK coefficients that the OPSC writer prints into opensbli.cpp,
code_generation/opsc.py:253-282).  It is plain data and serialises to JSON, so plans lowered
from the reference's problem scripts can be stored and run where the reference is not installed.
"""
import dataclasses
import json
import math
from typing import List, Optional, Tuple

# 2-register RK3 coefficients of RungeKutta(3) (schemes/temporal/rk_sbli.py:59-60)
RK3_RKOLD = (1.0 / 4.0, 3.0 / 20.0, 3.0 / 5.0)
RK3_RKNEW = (2.0 / 3.0, 5.0 / 12.0, 3.0 / 5.0)


@dataclasses.dataclass
class Plan:
    ndim: int = 3
    n: Tuple[int, int, int] = (64, 64, 64)
    delta: Tuple[float, float, float] = (2 * math.pi / 64,) * 3
    conv: str = "central_skew"      # central_skew | weno5js | teno5
    visc: str = "const"             # none | const | sutherland
    rk: str = "rk3"                 # rk3 (2-register) | ls_rk3
    precision: str = "fp64"         # fp64 | mixed
    bc: Tuple[Tuple[str, str], ...] = (("periodic", "periodic"),) * 3
    gama: float = 1.4
    Minf: float = 0.1
    Re: float = 1600.0
    Pr: float = 0.71
    weno_eps: float = 1e-6
    teno_ct: float = 1e-5
    teno_eps: float = 1e-15
    rk_a: Tuple[float, float, float] = RK3_RKOLD
    rk_b: Tuple[float, float, float] = RK3_RKNEW
    use_graphs: bool = True
    dt: Optional[float] = None
    niter: Optional[int] = None
    ic: str = "tgv"                 # tgv | host (evaluated from the script's initialisation kernel)
    name: str = ""
    kernels: List[str] = dataclasses.field(default_factory=list)  # the reference kernel names lowered

    @property
    def cells(self):
        return self.n[0] * self.n[1] * self.n[2]

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)

    def to_json(self):
        return json.dumps(dataclasses.asdict(self), indent=1)

    @classmethod
    def from_json(cls, s):
        d = json.loads(s)
        d["n"] = tuple(d["n"])
        d["delta"] = tuple(d["delta"])
        d["bc"] = tuple(tuple(x) for x in d["bc"])
        d["rk_a"] = tuple(d["rk_a"])
        d["rk_b"] = tuple(d["rk_b"])
        return cls(**d)


def tgv_plan(n=64, conv="central_skew", precision="fp64", Minf=0.1, Re=1600.0, Pr=0.71, gama=1.4, visc="const",
             dt=None, use_graphs=True):
    """3D Taylor-Green vortex on the periodic box [0, 2 pi)^3 with n^3 points (delta = 2 pi / n), the
    configuration of apps/taylor_green_vortex/taylor_green_vortex.py (conv='central_skew') and of the
    WENO5-JS variant (conv='weno5js')."""
    ns = (n, n, n) if isinstance(n, int) else tuple(n)
    return Plan(n=ns, delta=tuple(2 * math.pi / k for k in ns), conv=conv, visc=visc, precision=precision, Minf=Minf,
                Re=Re, Pr=Pr, gama=gama, dt=dt, use_graphs=use_graphs, ic="tgv",
                name="tgv_%s_%d" % (conv, ns[0]))


def tgv_cfl_dt(plan, cfl=0.5):
    """dt = cfl * min(delta) / max(|u| + a) of the TGV initial state (evaluated analytically at the
    grid points; the reference has a constant dt only, so it is computed once and fixed)."""
    import numpy as np
    g, M = plan.gama, plan.Minf
    idx = [np.arange(k) * d for k, d in zip(plan.n, plan.delta)]
    x0, x1, x2 = np.meshgrid(idx[0], idx[1], idx[2], indexing="ij")
    u0 = np.sin(x0) * np.cos(x1) * np.cos(x2)
    u1 = -np.cos(x0) * np.sin(x1) * np.cos(x2)
    p = 1.0 / (g * M * M) + (np.cos(2 * x0) + np.cos(2 * x1)) * (2 + np.cos(2 * x2)) / 16.0
    r = g * M * M * p
    a = np.sqrt(g * p / r)
    s = np.sqrt(u0 ** 2 + u1 ** 2) + a
    return cfl * min(plan.delta) / float(s.max())
