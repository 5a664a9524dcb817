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


def ls_rk3_ssp_coefficients(c=0.924574):
    """A and B of the 3-stage, 2-register (Williamson form) strong-stability-preserving RK3 with free
    parameter c = B1, as RungeKuttaLS(3, 'SSP') defines them (schemes/temporal/rk_LS.py:75-89, after
    Gottlieb, Shu and Tadmor, SIAM Review 43 (2001)).  Returns (A, B), A[0] = 0."""
    c2, c3, c4, c5, c6 = c ** 2, c ** 3, c ** 4, c ** 5, c ** 6
    z1 = math.sqrt(36 * c4 + 36 * c3 - 135 * c2 + 84 * c - 12)
    z2 = 2 * c2 + c - 2
    z3 = 12 * c4 - 18 * c3 + 18 * c2 - 11 * c + 2
    z4 = 36 * c4 - 36 * c3 + 13 * c2 - 8 * c + 4
    z5 = 69 * c3 - 62 * c2 + 28 * c - 8
    z6 = 34 * c4 - 46 * c3 + 34 * c2 - 13 * c + 2
    w = 3 * z2 - z1
    B = (c, (12 * c * (c - 1) * w - w ** 2) / (144 * c * (3 * c - 2) * (c - 1) ** 2),
         (-24 * (3 * c - 2) * (c - 1) ** 2) / (w ** 2 - 12 * c * (c - 1) * w))
    A = (0.0, (-z1 * (6 * c2 - 4 * c + 1) + 3 * z3) / ((2 * c + 1) * z1 - 3 * (c + 2) * (2 * c - 1) ** 2),
         (-z1 * z4 + 108 * (2 * c - 1) * c5 - 3 * (2 * c - 1) * z5) /
         (24 * z1 * c * (c - 1) ** 4 + 72 * c * z6 + 72 * c6 * (2 * c - 13)))
    return A, B


@dataclasses.dataclass
class Plan:
    ndim: int = 3
    n: Tuple[int, int, int] = (64, 64, 64)
    delta: Tuple[float, float, float] = (2 * math.pi / 64,) * 3
    conv: str = "central_skew"      # central_skew | weno5js | weno5z | teno5 | teno6
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
    # adaptive TENO cut-off from the modified Ducros sensor (teno.py:430-443, shock_sensors.py:12-49):
    # C_T = 10^-floor(a1 - a2 g(theta)) per interface; sensor_eps regularises theta's denominator
    teno_adaptive: bool = False
    teno_a1: float = 10.5
    teno_a2: float = 4.5
    sensor_eps: float = 1e-12
    # mixed precision on 2D blocks: interfaces whose two points' pressures differ by more than this
    # factor (strong shocks) form their characteristic flux in FP64 arithmetic; 0 keeps all in FP32
    shock_fp64: float = 0.0
    # 3D wall-bounded blocks: the Dirichlet face keeps rhou2 and sets rhoE = state + rhou2^2/(2 rho);
    # body_force = (A, xF, yF, bta, omega) of BF = A exp(-((x0-xF)^2 + (x1-yF)^2)) cos(bta x2)
    # sin(omega dt iter) in the continuity equation (apps/transitional_SBLI/transitional_SBLI.py)
    dirichlet_ke: bool = False
    body_force: Optional[Tuple[float, ...]] = None
    # channel blocks (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py): visc="power" takes
    # mu = T^visc_exp; forcing = (c0, c1, c2) subtracts c_i from the momentum equations and c_j u_j
    # from the energy equation; x1_grid="tanh" clusters x1 at both walls (used by the oracle)
    visc_exp: float = 0.7
    forcing: Optional[Tuple[float, ...]] = None
    x1_grid: str = "sinh"           # sinh: Lx1 sinh(by eta)/sinh(by) | tanh: -tanh(stretch (1-2eta))/tanh(stretch)
    stretch: float = 1.7            # | uniform: a Cartesian 2D block (no metric terms)
    # 2D Euler blocks (apps/inviscid_shock_reflection/inviscid_shock.py): the average the characteristic
    # system is built from ("roe" | "simple", averaging.py) and the constant states of Dirichlet x0
    # faces (side 0, side 1; rho, rhou0, rhou1, rhoE)
    averaging: str = "roe"
    dirichlet_x0: Optional[Tuple[Tuple[float, ...], ...]] = None
    rk_a: Tuple[float, float, float] = RK3_RKOLD
    rk_b: Tuple[float, float, float] = RK3_RKNEW
    use_graphs: bool = True
    dt: Optional[float] = None
    niter: Optional[int] = None
    ic: str = "tgv"                 # tgv | host (evaluated from the script's initialisation kernel)
    # 2D wall-bounded blocks: wall temperature, Sutherland constants, Dirichlet face states switched
    # at x0 = dirichlet_x_switch, x1 stretching (used by the oracle; the GPU takes coordinates)
    Twall: float = 1.67619431
    SuthT: float = 110.4
    RefT: float = 288.0
    dirichlet_lo: Tuple[float, ...] = (1.00000596004, 1.00000268202, 0.00565001630205, 0.94644428042)
    dirichlet_hi: Tuple[float, ...] = (1.129734572, 1.0921171, -0.058866065, 1.0590824)
    dirichlet_x_switch: float = 40.0
    Lx1: float = 115.0
    by: float = 5.0
    # one-sided closure of the central first derivatives at each face of a 2D wall-bounded block,
    # [axis][side]: "reduced_access" (boundary_conditions/reduced_access_scheme.py) or "carpenter"
    # (boundary_conditions/Carpenter_scheme.py, the reference's default)
    closure: Tuple[Tuple[str, str], ...] = (("reduced_access", "reduced_access"),) * 2
    # the WENO5 non-linear filter after every full step (filters/WENO_filter.py): "none" or
    # "weno5_constant" (dissipation_sensor='Constant'); filter_control = shock_filter_control
    filter: str = "none"
    filter_control: float = 1.0
    name: str = ""
    kernels: List[str] = dataclasses.field(default_factory=list)  # the reference kernel names lowered

    @property
    def cells(self):
        return self.n[0] * self.n[1] * (self.n[2] if self.ndim == 3 else 1)

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)

    def to_json(self):
        return json.dumps(dataclasses.asdict(self), indent=1)

    @classmethod
    def from_json(cls, s):
        d = json.loads(s)
        for k in ("n", "delta", "rk_a", "rk_b", "dirichlet_lo", "dirichlet_hi", "body_force", "forcing"):
            if d.get(k) is not None:
                d[k] = tuple(d[k])
        d["bc"] = tuple(tuple(x) for x in d["bc"])
        if d.get("dirichlet_x0") is not None:
            d["dirichlet_x0"] = tuple(tuple(x) for x in d["dirichlet_x0"])
        if "closure" in d:
            d["closure"] = tuple(tuple(x) for x in d["closure"])
        return cls(**d)


def tgv_plan(n=64, conv="central_skew", precision="fp64", Minf=0.1, Re=1600.0, Pr=0.71, gama=1.4, visc="const",
             dt=None, use_graphs=True):
    """3D Taylor-Green vortex on the periodic box [0, 2 pi)^3 with n^3 points (delta = 2 pi / n), the
    configuration of apps/taylor_green_vortex/taylor_green_vortex.py (conv='central_skew') and of the
    WENO5-JS, WENO5-Z, TENO5 and TENO6 variants (conv='weno5js', 'weno5z', 'teno5', 'teno6'; TENO with
    the fixed cut-off C_T = 1e-5 and eps = 1e-15)."""
    ns = (n, n, n) if isinstance(n, int) else tuple(n)
    return Plan(n=ns, delta=tuple(2 * math.pi / k for k in ns), conv=conv, visc=visc, precision=precision, Minf=Minf,
                Re=Re, Pr=Pr, gama=gama, dt=dt, use_graphs=use_graphs, ic="tgv",
                weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
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


def sbli3d_plan(n0=128, n1=64, n2=16, precision="fp64", conv="teno5", dt=0.04, use_graphs=True, delta2=2.0,
                closure=(("reduced_access", "reduced_access"),) * 2):
    """3D span-periodic shock/boundary-layer block: the 2D configuration of katzer_plan with a periodic
    x2 axis of spacing delta2 (apps/transitional_SBLI/transitional_SBLI.py's block without its body
    force), the Dirichlet top face carrying rhou2 = 0."""
    A, B = ls_rk3_ssp_coefficients()
    lo, hi = Plan.dirichlet_lo, Plan.dirichlet_hi
    return Plan(ndim=3, n=(n0, n1, n2), delta=(400.0 / (n0 - 1), 115.0 / (n1 - 1), delta2), conv=conv,
                visc="sutherland", rk="ls_rk3", precision=precision,
                bc=(("inlet_pressure_extrapolate", "extrapolation"), ("isothermal_wall", "dirichlet"),
                    ("periodic", "periodic")),
                gama=1.4, Minf=2.0, Re=950.0, Pr=0.72, teno_ct=1e-5, teno_eps=1e-15, rk_a=A, rk_b=B, dt=dt,
                use_graphs=use_graphs, ic="host", closure=tuple(tuple(c) for c in closure),
                weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
                dirichlet_lo=tuple(lo[:3]) + (0.0, lo[3]), dirichlet_hi=tuple(hi[:3]) + (0.0, hi[3]),
                name="sbli3d_%s_%dx%dx%d" % (conv, n0, n1, n2))


def transitional_plan(n0=500, n1=200, n2=100, precision="fp64", dt=0.025, use_graphs=True):
    """The block of apps/transitional_SBLI/transitional_SBLI.py: Mach 1.5, Re = 750, Pr = 0.72,
    Twall = 1.38099733, Sutherland 110.4/202.17, domain 375 x 140 x 27.32 with x1 = 140 sinh(5 eta)/sinh(5),
    TENO6 with the cut-off adapted by the Ducros sensor (a1 = 9.5, a2 = 3.5, sensor epsilon 1e-12,
    TENO eps 1e-30), RungeKuttaLS(3), the shock generator's Dirichlet face switched at x0 = 20 (rhoE
    carrying the local spanwise kinetic energy) and the body force A = 2.5e-3, xF = 20, yF = 4,
    bta = 0.23, omega = 0.1011."""
    g, M = 1.4, 1.5
    pre = (1.0, 1.0, 0.004666540532088, 0.0, 1.293661681951063)  # the script's "%.15f" values
    post = (1.091364590640748, 1.046223246979973, -0.045679092340368002, 0.0, 1.399487006243074)
    return Plan(ndim=3, n=(n0, n1, n2), delta=(375.0 / (n0 - 1), 140.0 / (n1 - 1), 27.32 / n2), conv="teno6",
                visc="sutherland", rk="ls_rk3", precision=precision,
                bc=(("inlet_pressure_extrapolate", "extrapolation"), ("isothermal_wall", "dirichlet"),
                    ("periodic", "periodic")),
                gama=g, Minf=M, Re=750.0, Pr=0.72, Twall=1.3809973268575328, SuthT=110.4, RefT=202.17,
                teno_ct=1e-5, teno_eps=1e-30, rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0),
                rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt, use_graphs=use_graphs, ic="host",
                teno_adaptive=True, teno_a1=9.5, teno_a2=3.5, sensor_eps=1e-12, Lx1=140.0, by=5.0,
                dirichlet_lo=pre, dirichlet_hi=post, dirichlet_x_switch=20.0, dirichlet_ke=True,
                body_force=(2.5e-3, 20.0, 4.0, 0.23, 0.1011), name="transitional_%dx%dx%d" % (n0, n1, n2))


def channel_plan(n0=129, n1=129, n2=129, precision="fp64", dt=2e-4, use_graphs=True, conv="teno6"):
    """The block of apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py (statistics off):
    Re = 190.71, Minf = 0.0955, Pr = 0.7, gama = 1.4, Twall = 1, mu = T^0.7, the forcing c = (-1, 0, 0),
    domain 4 pi x 2 x 4 pi/3 periodic in x0 and x2 with isothermal walls on both x1 faces (Carpenter
    closures), x1 = -tanh(1.7 (1 - 2 eta))/tanh(1.7), LLFTeno(6) with C_T = 1e-7 and eps = 1e-15,
    RungeKuttaLS(3, 'SSP'); 129^3 points and dt = 2e-4 as the script sets them."""
    A, B = ls_rk3_ssp_coefficients()
    carp = (("carpenter", "carpenter"),) * 2
    return Plan(ndim=3, n=(n0, n1, n2), delta=(4 * math.pi / n0, 2.0 / (n1 - 1), (4 * math.pi / 3) / n2), conv=conv,
                visc="power", visc_exp=0.7, rk="ls_rk3", precision=precision,
                bc=(("periodic", "periodic"), ("isothermal_wall", "isothermal_wall"), ("periodic", "periodic")),
                gama=1.4, Minf=0.0955, Re=190.71, Pr=0.7, Twall=1.0, teno_ct=1e-7, teno_eps=1e-15,
                weno_eps=1e-14 if conv == "weno5z" else 1e-6, rk_a=A, rk_b=B, dt=dt, use_graphs=use_graphs,
                ic="host", closure=carp, forcing=(-1.0, 0.0, 0.0), x1_grid="tanh", stretch=1.7,
                name="channel_%s_%dx%dx%d" % (conv, n0, n1, n2))


def channel_initial_state(plan, halo=3):
    """The initial state of apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:167-199 on a
    channel_plan block, halos included: x1 = -tanh(stretch (1 - 2 j/(n1-1)))/tanh(stretch), the mean
    velocity (1 - |x1|) Re where that is below 10 and 2.5 log((1 - |x1|) Re) + 5.5 elsewhere, plus the
    script's sinusoidal perturbations of amplitude 0.1 (2.5 log(Re) + 5.5); rho = 1, p = 1/(gama Minf^2).
    The box lengths are n0 delta0 (4 pi) and n2 delta2 (4 pi / 3).  Returns (q, x1): FP64
    [5][n2+2h][n1+2h][n0+2h] and the coordinate line [n1+2h]."""
    import numpy as np
    n0, n1, n2 = plan.n
    h = int(halo)
    lx, lz = n0 * plan.delta[0], n2 * plan.delta[2]
    j = np.arange(-h, n1 + h, dtype=np.float64)
    y1 = -np.tanh(plan.stretch * (1.0 - 2.0 * j / (n1 - 1.0))) / np.tanh(plan.stretch)
    x = (np.arange(-h, n0 + h) * plan.delta[0])[None, None, :]
    y = y1[None, :, None]
    z = (np.arange(-h, n2 + h) * plan.delta[2])[:, None, None]
    Re, b, kv = plan.Re, 5.5, 2.5
    wall = (1.0 - np.abs(y)) * Re
    with np.errstate(invalid="ignore", divide="ignore"):
        ubar = np.where(wall < 10.0, wall, kv * np.log(wall) + b)
    amp = 0.1 * (kv * np.log(Re) + b)
    sx, sy, sz = np.sin(4.0 * np.pi * x / lx), np.sin(np.pi * y), np.sin(2.0 * np.pi * z / lz)
    cx, cy, cz = np.cos(4.0 * np.pi * x / lx), 1.0 + np.cos(np.pi * y), np.cos(2.0 * np.pi * z / lz)
    u = ubar + amp * (lx / 2.0) * cx * sy * sz
    v = -amp * sx * cy * sz
    w = -amp * (lz / 2.0) * sx * sy * cz
    shape = (n2 + 2 * h, n1 + 2 * h, n0 + 2 * h)
    u, v, w = (np.broadcast_to(a, shape) for a in (u, v, w))
    p = 1.0 / (plan.gama * plan.Minf ** 2)
    q = np.stack([np.ones(shape), u, v, w, p / (plan.gama - 1.0) + 0.5 * (u * u + v * v + w * w)])
    return np.ascontiguousarray(q), y1


def shock_reflection_plan(n0=457, n1=255, precision="fp64", dt=0.1, use_graphs=True, conv="weno5z",
                          averaging="simple"):
    """The 2D inviscid shock reflection of apps/inviscid_shock_reflection/inviscid_shock.py: Euler
    equations at Mach 2 (gama = 1.4) on 350 x 115 with a uniform grid, LLFWeno(5, 'Z') with
    SimpleAverage, RungeKuttaLS(3); a Dirichlet inlet (the free stream) at x0 = 0, extrapolation at the
    outlet, a symmetry face at x1 = 0 and the shock generator's Dirichlet face at x1 = 115 (post-shock
    state where x0 >= 40; pressures as the script formats them, "%f").  457 x 255 and dt = 0.1 as the
    script sets them."""
    g, M = 1.4, 2.0

    def state(d, u0, u1, p):  # the generated code's rhoE = p/(gama-1) + d |u|^2 / 2
        return (d, d * u0, d * u1, (1.0 / (g - 1.0)) * p + 0.5 * d * (u0 ** 2 + u1 ** 2))
    free = state(1.0, 1.0, 0.0, 1.0 * (1.0 / g) * (1.0 / M ** 2))
    pre = state(1.0, 1.0, 0.0, float("%f" % (1.0 / (1.4 * 4.0))))
    post = state(1.129734572, 0.9667023804242755, -0.052106102140246795, float("%f" % (1.0 / (1.4 * 4.0) * 1.18646663)))
    return Plan(ndim=2, n=(n0, n1, 1), delta=(350.0 / (n0 - 1), 115.0 / (n1 - 1), 1.0), conv=conv, visc="none",
                rk="ls_rk3", precision=precision, averaging=averaging,
                bc=(("dirichlet", "extrapolation"), ("symmetry", "dirichlet"), ("periodic", "periodic")),
                gama=g, Minf=M, weno_eps=1e-14 if conv == "weno5z" else 1e-6, rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0),
                rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt, use_graphs=use_graphs, ic="host",
                x1_grid="uniform", dirichlet_x0=(free, (0.0, 0.0, 0.0, 0.0)), dirichlet_lo=pre, dirichlet_hi=post,
                dirichlet_x_switch=math.nextafter(40.0, 0.0), name="shock_reflection_%s_%dx%d" % (conv, n0, n1))


def euler_wave_plan(n0=400, n1=400, precision="fp64", dt=1e-3, use_graphs=True, conv="weno5z", averaging="simple"):
    """The 2D Euler density wave of apps/euler_wave/euler_wave.py: gama = 1.4 on the doubly periodic
    [0, 2)^2 (delta = 2/n), LLFWeno(5, 'Z') with SimpleAverage, RungeKutta(3) (two registers); the
    initial state rho = 1 + 0.2 sin(pi (x0 + x1)), u = (1, -0.5), p = 1 is advected unchanged by the
    Euler equations.  400 x 400 and dt = 1e-3 as the script sets them."""
    return Plan(ndim=2, n=(n0, n1, 1), delta=(2.0 / n0, 2.0 / n1, 1.0), conv=conv, visc="none", rk="rk3",
                precision=precision, averaging=averaging, bc=(("periodic", "periodic"),) * 3, gama=1.4,
                weno_eps=1e-14 if conv == "weno5z" else 1e-6, dt=dt, use_graphs=use_graphs, ic="host",
                x1_grid="uniform", name="euler_wave_%s_%dx%d" % (conv, n0, n1))


def viscous_shock_tube_plan(n0=500, n1=250, precision="fp64", dt=5e-6, use_graphs=True, conv="teno5"):
    """The 2D viscous shock tube of apps/viscous_shock_tube/viscous_shock_tube.py: Navier-Stokes with the
    constant viscosity mu = 1, Re = 200, Pr = 0.73, Minf = 1, gama = 1.4 on [0, 1] x [0, 0.5] (uniform),
    LLFTeno(5) with RoeAverage (C_T = 1e-6, eps = 1e-15), StoreSome central derivatives, RungeKuttaLS(3),
    adiabatic walls at x0 = 0, x0 = 1 and x1 = 0 with ReducedAccess closures and a symmetry face at x1 =
    0.5, whose derivatives stay central over its mirrored halos; 500 x 250 and dt = 5e-6 as the script
    sets them."""
    return Plan(ndim=2, n=(n0, n1, 1), delta=(1.0 / (n0 - 1), 0.5 / (n1 - 1), 1.0), conv=conv, visc="const",
                rk="ls_rk3", precision=precision, bc=(("adiabatic_wall", "adiabatic_wall"),
                                                      ("adiabatic_wall", "symmetry"), ("periodic", "periodic")),
                gama=1.4, Minf=1.0, Re=200.0, Pr=0.73, teno_ct=1e-6, teno_eps=1e-15,
                weno_eps=1e-14 if conv == "weno5z" else 1e-6, rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0),
                rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt, use_graphs=use_graphs, ic="host", x1_grid="uniform",
                closure=(("reduced_access", "reduced_access"), ("reduced_access", "none")),
                name="viscous_shock_tube_%dx%d" % (n0, n1))


def laminar_channel_plan(n0=16, n1=64, precision="fp64", dt=2e-4, use_graphs=True):
    """The 2D laminar channel of apps/channel_flow/laminar_2D/laminar_channel.py: central skew-symmetric
    convective terms (Skew) with StoreSome central viscous terms, Sutherland viscosity (110.4/273),
    Re = 90, Minf = 0.1, Pr = 0.72, the forcing c = (-1, 0), periodic x0 of length 2 pi, isothermal
    walls (Twall = 1) at x1 = -1 and x1 = 1 with Carpenter closures, a uniform grid, RungeKuttaLS(3);
    16 x 64 and dt = 2e-4 as the script sets them."""
    return Plan(ndim=2, n=(n0, n1, 1), delta=(2 * math.pi / n0, 2.0 / (n1 - 1), 1.0), conv="central_skew",
                visc="sutherland", rk="ls_rk3", precision=precision,
                bc=(("periodic", "periodic"), ("isothermal_wall", "isothermal_wall"), ("periodic", "periodic")),
                gama=1.4, Minf=0.1, Re=90.0, Pr=0.72, Twall=1.0, SuthT=110.4, RefT=273.0,
                rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0), rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt,
                use_graphs=use_graphs, ic="host", x1_grid="uniform", forcing=(-1.0, 0.0),
                closure=(("none", "none"), ("carpenter", "carpenter")), name="laminar_channel_%dx%d" % (n0, n1))


def _euler1d_state(g, d, u0, p):
    """rho, rhou0, rhoE as the generated 1D face kernels form them: rhoE = d u0^2 / 2 + p / (gama - 1)."""
    return (d, d * u0, 0.5 * d * u0 ** 2 + p / (g - 1.0))


def sod_plan(n0=200, precision="fp64", dt=2e-4, use_graphs=True, conv="teno5", averaging="roe"):
    """The Sod shock tube of apps/Sod_shock_tube/Sod_shock_tube.py: 1D Euler, gama = 1.4, [0, 1] with
    n0 points, LLFTeno(5) with RoeAverage (C_T = 1e-5, eps = 1e-16), RungeKuttaLS(3), Dirichlet faces
    holding the left (1, 0, 1) and right (0.125, 0, 0.1) states (rho, u, p); 200 points and dt = 2e-4
    as the script sets them."""
    g = 1.4
    return Plan(ndim=1, n=(n0, 1, 1), delta=(1.0 / (n0 - 1), 1.0, 1.0), conv=conv, visc="none", rk="ls_rk3",
                precision=precision, averaging=averaging, bc=(("dirichlet", "dirichlet"),) + (("periodic", "periodic"),) * 2,
                gama=g, teno_ct=1e-5, teno_eps=1e-16, weno_eps=1e-14 if conv == "weno5z" else 1e-6,
                rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0), rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt,
                use_graphs=use_graphs, ic="host", x1_grid="uniform",
                dirichlet_x0=(_euler1d_state(g, 1.0, 0.0, 1.0), _euler1d_state(g, 0.125, 0.0, 0.1)),
                name="sod_%s_%d" % (conv, n0))


def shu_osher_plan(n0=3200, precision="fp64", dt=2e-4, use_graphs=True, conv="weno5z", averaging="roe"):
    """The Shu-Osher shock/entropy-wave interaction of apps/shu_osher/shu_osher.py: 1D Euler, gama = 1.4,
    [-5, 5] with n0 points, LLFWeno(5, 'Z') with RoeAverage, RungeKuttaLS(3), Dirichlet faces holding
    the post-shock state (3.857143, 2.629369, 10.33333) and (1 + 0.2 sin(25), 0, 1) (rho, u, p); 3200
    points and dt = 2e-4 as the script sets them."""
    import math as m
    g = 1.4
    return Plan(ndim=1, n=(n0, 1, 1), delta=(10.0 / (n0 - 1), 1.0, 1.0), conv=conv, visc="none", rk="ls_rk3",
                precision=precision, averaging=averaging, bc=(("dirichlet", "dirichlet"),) + (("periodic", "periodic"),) * 2,
                gama=g, Minf=0.1, teno_ct=1e-5, teno_eps=1e-15, weno_eps=1e-14 if conv == "weno5z" else 1e-6,
                rk_a=(0.0, -5.0 / 9.0, -153.0 / 128.0), rk_b=(1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0), dt=dt,
                use_graphs=use_graphs, ic="host", x1_grid="uniform",
                dirichlet_x0=(_euler1d_state(g, 3.857143, 2.629369, 10.33333),
                              _euler1d_state(g, 1.0 + 0.2 * m.sin(5 * 5.0), 0.0, 1.0)),
                name="shu_osher_%s_%d" % (conv, n0))


def katzer_plan(n0=512, n1=256, precision="fp64", conv="teno5", dt=0.04, use_graphs=True, adaptive=False,
                closure=(("reduced_access", "reduced_access"),) * 2):
    """2D laminar shock-wave/boundary-layer interaction (apps/katzer_SBLI/katzer_SBLI.py constants):
    Mach 2, Re = 950, Pr = 0.72, Twall = 1.67619431, Sutherland 110.4/288, TENO5 with C_T = 1e-5 and
    eps = 1e-15, domain [0, 400] x [0, 115] with x1 = 115 sinh(5 eta)/sinh(5), LS-RK3 (SSP).
    adaptive=True gives the script as published: the TENO cut-off adapted per interface by the
    modified Ducros sensor (a1 = 10.5, a2 = 4.5, sensor epsilon 1e-12).  closure[axis][side] names
    each face's one-sided derivative closure (the script sets ReducedAccess on all four)."""
    A, B = ls_rk3_ssp_coefficients()
    return Plan(ndim=2, n=(n0, n1, 1), delta=(400.0 / (n0 - 1), 115.0 / (n1 - 1), 1.0), conv=conv, visc="sutherland",
                rk="ls_rk3", precision=precision,
                bc=(("inlet_pressure_extrapolate", "extrapolation"), ("isothermal_wall", "dirichlet"),
                    ("periodic", "periodic")),
                gama=1.4, Minf=2.0, Re=950.0, Pr=0.72, teno_ct=1e-5, teno_eps=1e-15, rk_a=A, rk_b=B, dt=dt,
                use_graphs=use_graphs, ic="host", teno_adaptive=adaptive,
                closure=tuple(tuple(c) for c in closure),
                name="katzer_%s%s_%dx%d" % (conv, "_adaptive" if adaptive else "", n0, n1))
