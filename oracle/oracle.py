"""ctypes front-end to the C restatement in oracle/src (test infrastructure only).

build() compiles oracle/src/osb_oracle.c with gcc into oracle/_build/libosb_oracle.so; the
functions below wrap its entry points with numpy arrays laid out [var][z][y][x].
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libosb_oracle.so")

CONV = {"central_skew": 0, "weno5js": 1, "teno5": 2, "weno5z": 3, "teno6": 4}
VISC = {"none": 0, "const": 1, "sutherland": 2}
RK = {"rk3": 0, "ls_rk3_ssp": 1}
BC = {"periodic": 0, "symmetry": 1}


class Cfg(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("delta", ctypes.c_double * 3),
        ("gama", ctypes.c_double),
        ("Minf", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("conv", ctypes.c_int),
        ("visc", ctypes.c_int),
        ("rk", ctypes.c_int),
        ("bc", (ctypes.c_int * 2) * 3),
        ("teno_ct", ctypes.c_double),
        ("teno_eps", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("filter", ctypes.c_int),
        ("filter_control", ctypes.c_double),
        ("teno_adaptive", ctypes.c_int),
        ("teno_a1", ctypes.c_double),
        ("teno_a2", ctypes.c_double),
        ("sensor_eps", ctypes.c_double),
    ]


FILTER = {"none": 0, "weno5_constant": 1}


def build(force=False):
    srcs = [os.path.join(HERE, "src", f) for f in ("osb_oracle.c", "osb_oracle1d.c", "osb_oracle2d.c", "osb_oracle3w.c")]
    deps = srcs + [os.path.join(HERE, "src", "osb_oracle.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-o", tmp] + srcs + ["-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        for name in ("osbo_tgv_init", "osbo_run", "osbo_residual", "osbo_cutoff", "osbo2d_run", "osbo2d_metrics",
                     "osbo2d_cutoff", "osbo3w_run", "osbo3w_residual"):
            getattr(_lib, name).restype = ctypes.c_int
    return _lib


def make_cfg(n, delta, gama=1.4, Minf=0.1, Re=1600.0, Pr=0.71, conv="central_skew", visc="const", rk="rk3",
             bc="periodic", dt=5e-3, teno_ct=1e-5, teno_eps=1e-15, filter="none", filter_control=1.0,
             teno_adaptive=False, teno_a1=10.5, teno_a2=4.5, sensor_eps=1e-12):
    c = Cfg()
    c.ndim = len(n) if len(n) == 2 else 3
    nn = list(n) + [1] * (3 - len(n))
    dd = list(delta) + [1.0] * (3 - len(delta))
    for i in range(3):
        c.n[i] = nn[i]
        c.delta[i] = dd[i]
    c.gama, c.Minf, c.Re, c.Pr = gama, Minf, Re, Pr
    c.conv, c.visc, c.rk = CONV[conv], VISC[visc], RK[rk]
    for d in range(3):
        for s in range(2):
            c.bc[d][s] = BC[bc if isinstance(bc, str) else bc[d][s]]
    c.teno_ct, c.teno_eps, c.dt = teno_ct, teno_eps, dt
    c.filter, c.filter_control = FILTER[filter], filter_control
    c.teno_adaptive = 1 if teno_adaptive else 0
    c.teno_a1, c.teno_a2, c.sensor_eps = teno_a1, teno_a2, sensor_eps
    return c


def _shape(c):
    nv = 5 if c.ndim == 3 else 4
    return (nv, c.n[2], c.n[1], c.n[0])


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def tgv_init(c):
    q = np.zeros(_shape(c), dtype=np.float64)
    assert lib().osbo_tgv_init(ctypes.byref(c), _ptr(q)) == 0
    return q


def run(c, q0, nsteps, with_ke=False):
    q = np.ascontiguousarray(q0, dtype=np.float64).copy()
    ke = np.zeros(nsteps + 1, dtype=np.float64)
    rc = lib().osbo_run(ctypes.byref(c), _ptr(q), int(nsteps), _ptr(ke) if with_ke else None)
    assert rc == 0, rc
    return (q, ke) if with_ke else q


def residual(c, q0):
    q = np.ascontiguousarray(q0, dtype=np.float64)
    r = np.zeros_like(q)
    assert lib().osbo_residual(ctypes.byref(c), _ptr(q), _ptr(r)) == 0
    return r


def cutoff(c, q0):
    """Adaptive TENO cut-off C_T of the interior state q0 [5][n2][n1][n0] on a 3D block, laid out
    [n2][n1][n0] (the reference's TENO_B0 field; osb_oracle.c ducros_sensor / teno_cutoff3)."""
    q = np.ascontiguousarray(q0, dtype=np.float64)
    ct = np.zeros(q.shape[1:], dtype=np.float64)
    assert lib().osbo_cutoff(ctypes.byref(c), _ptr(q), _ptr(ct)) == 0
    return ct


class Cfg2D(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int * 2),
        ("delta", ctypes.c_double * 2),
        ("gama", ctypes.c_double),
        ("Minf", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("Twall", ctypes.c_double),
        ("SuthT", ctypes.c_double),
        ("RefT", ctypes.c_double),
        ("teno_eps", ctypes.c_double),
        ("teno_ct", ctypes.c_double),
        ("Lx1", ctypes.c_double),
        ("by", ctypes.c_double),
        ("rkA", ctypes.c_double * 3),
        ("rkB", ctypes.c_double * 3),
        ("dt", ctypes.c_double),
        ("teno_adaptive", ctypes.c_int),
        ("teno_a1", ctypes.c_double),
        ("teno_a2", ctypes.c_double),
        ("sensor_eps", ctypes.c_double),
        ("closure", (ctypes.c_int * 2) * 2),
        ("conv", ctypes.c_int),
        ("euler", ctypes.c_int),
        ("simple_avg", ctypes.c_int),
        ("bc", (ctypes.c_int * 2) * 2),
        ("face0", (ctypes.c_double * 4) * 2),
        ("top", (ctypes.c_double * 4) * 2),
        ("x_switch", ctypes.c_double),
        ("rk2reg", ctypes.c_int),
        ("cartesian", ctypes.c_int),
        ("visc_const", ctypes.c_int),
        ("skew", ctypes.c_int),
        ("force", ctypes.c_double * 2),
    ]


CLOSURES = {"reduced_access": 0, "carpenter": 1, "none": 2}


def make_cfg2d(plan):
    """Oracle configuration from a 2D Plan (opensbli_gb300.plan.Plan with ndim=2)."""
    c = Cfg2D()
    for d in range(2):
        c.n[d] = plan.n[d]
        c.delta[d] = plan.delta[d]
    c.gama, c.Minf, c.Re, c.Pr = plan.gama, plan.Minf, plan.Re, plan.Pr
    c.Twall, c.SuthT, c.RefT = plan.Twall, plan.SuthT, plan.RefT
    c.teno_eps, c.teno_ct = plan.teno_eps, plan.teno_ct
    c.Lx1, c.by = plan.Lx1, plan.by
    for s in range(3):
        c.rkA[s] = plan.rk_a[s]
        c.rkB[s] = plan.rk_b[s]
    c.dt = plan.dt
    c.teno_adaptive = 1 if getattr(plan, "teno_adaptive", False) else 0
    c.teno_a1 = getattr(plan, "teno_a1", 10.5)
    c.teno_a2 = getattr(plan, "teno_a2", 4.5)
    c.sensor_eps = getattr(plan, "sensor_eps", 1e-30)
    for d in range(2):
        for side in range(2):
            c.closure[d][side] = CLOSURES[plan.closure[d][side]]
    c.conv = CONV[plan.conv]
    # Euler blocks: Cartesian x1, no viscous terms, the faces and states of the plan
    c.euler = 1 if plan.visc == "none" else 0
    c.simple_avg = 1 if plan.averaging == "simple" else 0
    kinds = {"dirichlet": 1, "symmetry": 2, "periodic": 3, "adiabatic_wall": 4}
    c.rk2reg = 1 if plan.rk == "rk3" else 0
    c.cartesian = 1 if plan.x1_grid == "uniform" else 0
    c.visc_const = 1 if plan.visc == "const" else 0
    for d in range(2):
        for side in range(2):
            c.bc[d][side] = kinds.get(plan.bc[d][side], 0) if (c.euler or c.cartesian) else 0
    if c.cartesian and plan.bc[1][1] == "isothermal_wall":
        c.bc[1][1] = 5  # the channel's second wall
    c.skew = 1 if plan.conv == "central_skew" else 0
    for d, f in enumerate((plan.forcing or (0.0, 0.0))[:2]):
        c.force[d] = f
    for side, st in enumerate(plan.dirichlet_x0 or ()):
        for v in range(4):
            c.face0[side][v] = st[v]
    if c.euler and plan.bc[1][1] == "dirichlet":
        for v in range(4):
            c.top[0][v] = plan.dirichlet_lo[v]
            c.top[1][v] = plan.dirichlet_hi[v]
        c.x_switch = plan.dirichlet_x_switch
    return c


def residual2d(plan, q0_padded):
    """Right-hand side [4][n1][n0] of a padded FP64 state (boundary conditions applied first)."""
    c = make_cfg2d(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64)
    assert q.shape == (4, plan.n[1] + 8, plan.n[0] + 8)
    r = np.zeros((4, plan.n[1], plan.n[0]))
    assert lib().osbo2d_residual(ctypes.byref(c), _ptr(q), _ptr(r)) == 0
    return r


def carpenter_d1():
    """The oracle's Carpenter first-derivative closure weights, [4][6] (weight of f(m) at point r)."""
    out = np.zeros(24)
    lib().osbo2d_carpenter_d1(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out.reshape(4, 6)


def run2d(plan, q0_padded, nsteps):
    """q0_padded: FP64 [4][n1+8][n0+8] with a 4-point halo.  Returns the state after nsteps."""
    c = make_cfg2d(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64).copy()
    assert q.shape == (4, plan.n[1] + 8, plan.n[0] + 8)
    assert lib().osbo2d_run(ctypes.byref(c), _ptr(q), int(nsteps)) == 0
    return q


def cutoff2d(plan, q0_padded):
    """The adaptive TENO cut-off [n1][n0] of a padded FP64 state (boundary conditions applied)."""
    c = make_cfg2d(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64)
    assert q.shape == (4, plan.n[1] + 8, plan.n[0] + 8)
    ct = np.zeros((plan.n[1], plan.n[0]))
    assert lib().osbo2d_cutoff(ctypes.byref(c), _ptr(q), _ptr(ct)) == 0
    return ct


def metrics2d(plan):
    c = make_cfg2d(plan)
    D = np.zeros((plan.n[1], plan.n[0]))
    S = np.zeros_like(D)
    assert lib().osbo2d_metrics(ctypes.byref(c), _ptr(D), _ptr(S)) == 0
    return D, S


class Cfg1D(ctypes.Structure):
    _fields_ = [
        ("n0", ctypes.c_int),
        ("delta0", ctypes.c_double),
        ("gama", ctypes.c_double),
        ("conv", ctypes.c_int),
        ("teno_eps", ctypes.c_double),
        ("teno_ct", ctypes.c_double),
        ("simple_avg", ctypes.c_int),
        ("rkA", ctypes.c_double * 3),
        ("rkB", ctypes.c_double * 3),
        ("dt", ctypes.c_double),
        ("bc1", ctypes.c_int),
        ("face", (ctypes.c_double * 3) * 2),
    ]


def make_cfg1d(plan):
    """Oracle configuration from a 1D Plan (osb_oracle1d.c)."""
    c = Cfg1D()
    c.n0, c.delta0, c.gama = plan.n[0], plan.delta[0], plan.gama
    c.conv = CONV[plan.conv]
    c.teno_eps, c.teno_ct = plan.teno_eps, plan.teno_ct
    c.simple_avg = 1 if plan.averaging == "simple" else 0
    for s in range(3):
        c.rkA[s] = plan.rk_a[s]
        c.rkB[s] = plan.rk_b[s]
    c.dt = plan.dt
    c.bc1 = 1 if plan.bc[0][1] == "extrapolation" else 0
    for side, st in enumerate(plan.dirichlet_x0 or ()):
        for v in range(3):
            c.face[side][v] = st[v]
    return c


def run1d(plan, q0_padded, nsteps):
    """q0_padded: FP64 [3][n0+8] with a 4-point halo.  Returns the state after nsteps."""
    c = make_cfg1d(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64).copy()
    assert q.shape == (3, plan.n[0] + 8)
    assert lib().osbo1d_run(ctypes.byref(c), _ptr(q), int(nsteps)) == 0
    return q


def residual1d(plan, q0_padded):
    c = make_cfg1d(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64)
    r = np.zeros((3, plan.n[0]))
    assert lib().osbo1d_residual(ctypes.byref(c), _ptr(q), _ptr(r)) == 0
    return r


class Cfg3W(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int * 3),
        ("delta", ctypes.c_double * 3),
        ("gama", ctypes.c_double),
        ("Minf", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("Twall", ctypes.c_double),
        ("SuthT", ctypes.c_double),
        ("RefT", ctypes.c_double),
        ("teno_eps", ctypes.c_double),
        ("teno_ct", ctypes.c_double),
        ("Lx1", ctypes.c_double),
        ("by", ctypes.c_double),
        ("rkA", ctypes.c_double * 3),
        ("rkB", ctypes.c_double * 3),
        ("dt", ctypes.c_double),
        ("closure", (ctypes.c_int * 2) * 2),
        ("conv", ctypes.c_int),
        ("dirichlet", (ctypes.c_double * 5) * 2),
        ("x_switch", ctypes.c_double),
        ("dirichlet_ke", ctypes.c_int),
        ("bf_A", ctypes.c_double),
        ("bf_xF", ctypes.c_double),
        ("bf_yF", ctypes.c_double),
        ("bf_bta", ctypes.c_double),
        ("bf_omega", ctypes.c_double),
        ("teno_adaptive", ctypes.c_int),
        ("teno_a1", ctypes.c_double),
        ("teno_a2", ctypes.c_double),
        ("sensor_eps", ctypes.c_double),
        ("periodic0", ctypes.c_int),
        ("wall1", ctypes.c_int),
        ("grid_tanh", ctypes.c_int),
        ("stretch", ctypes.c_double),
        ("visc_pow", ctypes.c_double),
        ("force", ctypes.c_double * 3),
    ]


def make_cfg3w(plan):
    """Oracle configuration from a 3D wall-bounded Plan (span-periodic x2; osb_oracle3w.c)."""
    c = Cfg3W()
    for d in range(3):
        c.n[d] = plan.n[d]
        c.delta[d] = plan.delta[d]
    c.gama, c.Minf, c.Re, c.Pr = plan.gama, plan.Minf, plan.Re, plan.Pr
    c.Twall, c.SuthT, c.RefT = plan.Twall, plan.SuthT, plan.RefT
    c.teno_eps, c.teno_ct = plan.teno_eps, plan.teno_ct
    c.Lx1, c.by = plan.Lx1, plan.by
    for s in range(3):
        c.rkA[s] = plan.rk_a[s]
        c.rkB[s] = plan.rk_b[s]
    c.dt = plan.dt
    for d in range(2):
        for side in range(2):
            c.closure[d][side] = CLOSURES[plan.closure[d][side]]
    c.conv = CONV[plan.conv]
    if plan.bc[1][1] == "dirichlet":
        for v in range(5):
            c.dirichlet[0][v] = plan.dirichlet_lo[v]
            c.dirichlet[1][v] = plan.dirichlet_hi[v]
    c.x_switch = plan.dirichlet_x_switch
    c.dirichlet_ke = 1 if getattr(plan, "dirichlet_ke", False) else 0
    bf = getattr(plan, "body_force", None) or (0.0, 0.0, 0.0, 0.0, 0.0)
    c.bf_A, c.bf_xF, c.bf_yF, c.bf_bta, c.bf_omega = bf
    c.teno_adaptive = 1 if getattr(plan, "teno_adaptive", False) else 0
    c.teno_a1, c.teno_a2 = getattr(plan, "teno_a1", 10.5), getattr(plan, "teno_a2", 4.5)
    c.sensor_eps = getattr(plan, "sensor_eps", 1e-12)
    c.periodic0 = 1 if plan.bc[0][0] == "periodic" else 0
    c.wall1 = 1 if plan.bc[1][1] == "isothermal_wall" else 0
    c.grid_tanh = 1 if plan.x1_grid == "tanh" else 0
    c.stretch = plan.stretch
    c.visc_pow = plan.visc_exp if plan.visc == "power" else 0.0
    for d, f in enumerate(plan.forcing or (0.0, 0.0, 0.0)):
        c.force[d] = f
    return c


def run3w(plan, q0_padded, nsteps):
    """q0_padded: FP64 [5][n2+8][n1+8][n0+8] with a 4-point halo.  Returns the state after nsteps."""
    c = make_cfg3w(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64).copy()
    assert q.shape == (5, plan.n[2] + 8, plan.n[1] + 8, plan.n[0] + 8)
    assert lib().osbo3w_run(ctypes.byref(c), _ptr(q), int(nsteps)) == 0
    return q


def residual3w(plan, q0_padded):
    """Right-hand side [5][n2][n1][n0] of a padded FP64 state (boundary conditions applied first)."""
    c = make_cfg3w(plan)
    q = np.ascontiguousarray(q0_padded, dtype=np.float64)
    r = np.zeros((5, plan.n[2], plan.n[1], plan.n[0]))
    assert lib().osbo3w_residual(ctypes.byref(c), _ptr(q), _ptr(r)) == 0
    return r
