"""GB300Writer: lowering of the reference's own problem scripts, plan serialisation."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from opensbli_gb300.plan import Plan, tgv_plan, tgv_cfl_dt
from opensbli_gb300.writer import _eval_c_expr
from helpers import GOLDEN, golden_plan

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "oracle", "gen"))
from refpath import default_ref  # noqa: E402

REF = default_ref()


def test_plan_json_roundtrip():
    p = tgv_plan(48, conv="weno5js", precision="mixed", Minf=1.25)
    q = Plan.from_json(p.to_json())
    assert q == p


def test_golden_plans_are_what_the_kernels_implement():
    c = golden_plan("tgv_central")
    assert (c.conv, c.visc, c.rk) == ("central_skew", "const", "rk3")
    assert c.bc == (("periodic", "periodic"),) * 3
    assert c.rk_a == (0.25, 0.15, 0.6) and abs(c.rk_b[0] - 2 / 3) < 1e-16
    assert c.n == (64, 64, 64) and abs(c.delta[0] - 2 * math.pi / 64) < 1e-15
    assert (c.Re, c.Minf, c.Pr, c.gama) == (1600.0, 0.1, 0.71, 1.4)
    assert c.dt == 0.003385 and c.niter == 5909
    w = golden_plan("tgv_weno")
    assert w.conv == "weno5js" and w.visc == "const"
    s = golden_plan("tgsym_central")
    assert s.bc == (("symmetry", "symmetry"),) * 3 and s.Re == 800.0
    assert abs(s.delta[0] - math.pi / 32) < 1e-15


def test_value_expressions():
    env = {"block0np0": 64}
    assert abs(_eval_c_expr("2*M_PI/block0np0", env) - 2 * math.pi / 64) < 1e-15
    with pytest.raises(ValueError):
        _eval_c_expr("__import__('os')", env)


def test_katzer_plan_matches_lowered_script():
    from opensbli_gb300.plan import katzer_plan
    k = katzer_plan()
    g = golden_plan("katzer_teno")
    for f in ("ndim", "n", "conv", "visc", "rk", "bc", "gama", "Minf", "Re", "Pr", "Twall", "SuthT", "RefT", "teno_eps",
              "teno_ct", "dirichlet_lo", "dirichlet_hi", "dirichlet_x_switch", "Lx1", "by", "closure"):
        assert getattr(k, f) == getattr(g, f), f
    assert np.allclose(k.rk_a, g.rk_a, atol=1e-15) and np.allclose(k.rk_b, g.rk_b, rtol=1e-15)
    assert np.allclose(k.delta[:2], g.delta[:2], rtol=1e-15)


def test_published_katzer_script_lowers_to_adaptive_teno():
    from opensbli_gb300.plan import katzer_plan
    k = katzer_plan(adaptive=True)
    g = golden_plan("katzer_adaptive")
    assert g.teno_adaptive and not golden_plan("katzer_teno").teno_adaptive
    for f in ("conv", "teno_adaptive", "teno_a1", "teno_a2", "teno_eps", "bc", "Twall"):
        assert getattr(k, f) == getattr(g, f), f
    # the script substitutes epsilon = 1e-30, but the generated code keeps the value the sensor gives
    # its constant (the line is not `epsilon=Input;`), so the lowered plan does too
    assert g.sensor_eps == 1e-12 == k.sensor_eps
    assert "ConstituentRelations evaluation" in g.kernels


def test_3d_sensor_kernels_lower_to_adaptive_teno():
    """On 3D blocks the sensor's velocity derivatives are separate kernels ("ConstituentRelations CD
    u_i x_j") writing work arrays that the sensor kernel reads; the writer follows them to the
    adaptive cut-off, and the same TENO5 case without the sensor lowers to the fixed one."""
    g = golden_plan("tgv_teno_adaptive")
    assert g.teno_adaptive and g.conv == "teno5" and g.sensor_eps == 1e-12
    assert (g.teno_a1, g.teno_a2) == (10.5, 4.5)
    assert sum(k.startswith("ConstituentRelations CD u") for k in g.kernels) == 9
    assert not golden_plan("tgv_teno").teno_adaptive


def test_3d_wall_script_lowers_to_the_span_periodic_plan():
    """The 3D shock/boundary-layer script (periodic x2) lowers to the same plan as sbli3d_plan, and the
    writer's numpy evaluation of its initialisation kernel reproduces the reference's initial state
    (halos included) on the fixture's grid."""
    from opensbli_gb300.plan import sbli3d_plan
    g = golden_plan("sbli3d_teno")
    p = sbli3d_plan(*g.n)
    assert g.replace(kernels=[], name="", niter=None) == p.replace(kernels=[], name="")
    assert g.bc[2] == ("periodic", "periodic") and g.dirichlet_hi[3] == 0.0


def test_transitional_script_lowers_to_its_plan():
    """The transitional_SBLI block lowers with its adaptive TENO6 cut-off (metric sensor), body force
    and Dirichlet face carrying the spanwise kinetic energy, to the plan of transitional_plan."""
    from opensbli_gb300.plan import transitional_plan
    g = golden_plan("transitional_sbli")
    p = transitional_plan(*g.n)
    assert g.replace(kernels=[], name="", niter=None) == p.replace(kernels=[], name="")
    assert g.teno_adaptive and g.conv == "teno6" and g.dirichlet_ke and g.body_force == (2.5e-3, 20.0, 4.0, 0.23, 0.1011)


def test_shock_reflection_script_lowers_to_its_plan():
    """The inviscid shock reflection lowers to a Cartesian 2D Euler block with WENO5-Z, the simple
    average, a Dirichlet inlet, a symmetry face and the shock generator's Dirichlet face switched at
    x0 >= 40; the face states evaluated from the script's kernels equal shock_reflection_plan's to the
    last bit or two (high-precision evaluation against the generated code's double arithmetic)."""
    import math
    from opensbli_gb300.plan import shock_reflection_plan
    g = golden_plan("shock_reflection")
    p = shock_reflection_plan(*g.n[:2])
    states = ("dirichlet_x0", "dirichlet_lo", "dirichlet_hi")
    assert g.replace(kernels=[], name="", niter=None, **{k: None for k in states}) == \
        p.replace(kernels=[], name="", **{k: None for k in states})
    flat = lambda v: [x for t in v for x in (t if isinstance(t, tuple) else (t,))]
    for k in states:
        a, b = flat(getattr(g, k)), flat(getattr(p, k))
        assert len(a) == len(b) and all(math.isclose(x, y, rel_tol=1e-15, abs_tol=0) for x, y in zip(a, b)), k
    assert g.visc == "none" and g.averaging == "simple" and g.conv == "weno5z" and g.x1_grid == "uniform"
    assert g.dirichlet_x_switch == math.nextafter(40.0, 0.0)


def test_laminar_channel_script_lowers_to_its_plan():
    """The 2D laminar channel lowers with its skew-symmetric convective terms (one kernel, derivatives of
    products formed inline, checked by the physics check), forcing, periodic x0 and walls on both x1 faces."""
    from opensbli_gb300.plan import laminar_channel_plan
    g = golden_plan("laminar_channel")
    assert g.replace(kernels=[], name="", niter=None) == laminar_channel_plan(*g.n[:2]).replace(kernels=[], name="")
    assert g.conv == "central_skew" and g.forcing == (-1.0, 0.0)


def test_viscous_shock_tube_script_lowers_to_its_plan():
    """The viscous shock tube lowers to a Cartesian 2D block with the constant viscosity, adiabatic walls
    on three faces (ReducedAccess) and a symmetry top face without a one-sided closure."""
    from opensbli_gb300.plan import viscous_shock_tube_plan
    g = golden_plan("viscous_shock_tube")
    p = viscous_shock_tube_plan(*g.n[:2])
    assert g.replace(kernels=[], name="", niter=None) == p.replace(kernels=[], name="")
    assert g.visc == "const" and g.closure[1] == ("reduced_access", "none")


def test_euler_wave_script_lowers_to_its_plan():
    """The doubly periodic Euler wave lowers with its exchanges on both axes and RungeKutta(3)'s two
    registers (rkold, rknew) to euler_wave_plan's plan."""
    from opensbli_gb300.plan import euler_wave_plan
    g = golden_plan("euler_wave")
    assert g.replace(kernels=[], name="", niter=None) == euler_wave_plan(*g.n[:2]).replace(kernels=[], name="")
    assert g.rk == "rk3" and g.bc[:2] == (("periodic", "periodic"),) * 2


@pytest.mark.parametrize("case", ["sod", "shu_osher"])
def test_euler1d_scripts_lower_to_their_plans(case):
    """The Sod shock tube (TENO5) and the Shu-Osher problem (WENO5-Z) lower to 1D Euler blocks with
    Roe averaging and Dirichlet faces whose states the writer evaluates from the face kernels (the
    Shu-Osher outlet kernel reads its u0 before setting it: 0, as the generated code's locals start)."""
    from opensbli_gb300.plan import sod_plan, shu_osher_plan
    g = golden_plan(case)
    p = {"sod": sod_plan, "shu_osher": shu_osher_plan}[case](g.n[0])
    assert g.replace(kernels=[], name="", niter=None) == p.replace(kernels=[], name="")
    assert g.ndim == 1 and g.visc == "none" and g.averaging == "roe"


def test_channel_script_lowers_to_its_plan():
    """The channel script (compressible_TCF_TENO, statistics off) lowers with periodic x0, isothermal
    walls on both x1 faces, the power-law viscosity and the constant forcing, to channel_plan's plan."""
    from opensbli_gb300.plan import channel_plan
    g = golden_plan("channel_teno")
    p = channel_plan(*g.n)
    assert g.replace(kernels=[], name="", niter=None) == p.replace(kernels=[], name="")
    assert g.visc == "power" and g.visc_exp == 0.7 and g.forcing == (-1.0, 0.0, 0.0)
    assert g.bc[0] == ("periodic", "periodic") and g.bc[1] == ("isothermal_wall", "isothermal_wall")


def test_channel_initial_state_helper_matches_reference():
    """plan.channel_initial_state (the script's initial condition restated with numpy, for drivers that
    run without the reference) against the generated code's initial state, halos included."""
    from opensbli_gb300.plan import channel_plan, channel_initial_state
    d = np.load(os.path.join(GOLDEN, "ref_channel_teno.npz"))
    q, x1 = channel_initial_state(channel_plan(*(int(x) for x in d["n"])), halo=4)
    assert np.abs(x1 - d["x1"]).max() <= 1e-15
    err = [float(np.abs(q[v] - d["q0"][v]).max() / np.abs(d["q0"][v]).max()) for v in range(5)]
    assert max(err) <= 1e-13, err


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "opensbli")), reason="reference tree not present")
def test_channel_initial_state_matches_reference(tmp_path):
    """The channel's initial condition (laminar/log profile with sinusoidal perturbations) and its
    tanh-clustered coordinates, evaluated by the writer, against the generated code's."""
    r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", "channel_teno",
                        "--out", str(tmp_path), "--ref", REF, "--params", "block0np0=32,block0np1=24,block0np2=16"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(os.path.join(GOLDEN, "ref_channel_teno.npz"))
    ic = np.load(tmp_path / "ic.npy")
    ref = d["q0"][:, 4:-4, 4:-4, 4:-4]
    assert ic.shape == ref.shape
    assert np.abs(ic - ref).max() <= 1e-13 * np.abs(ref).max(), float(np.abs(ic - ref).max())


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "opensbli")), reason="reference tree not present")
def test_3d_wall_initial_state_matches_reference(tmp_path):
    import json
    r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", "sbli3d_teno",
                        "--out", str(tmp_path), "--ref", REF, "--params", "block0np0=32,block0np1=24,block0np2=8"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(os.path.join(GOLDEN, "ref_sbli3d_teno.npz"))
    ic = np.load(tmp_path / "ic.npy")
    ref = d["q0"][:, 4:-4, 4:-4, 4:-4]
    assert ic.shape == ref.shape
    # the profile is a 50-coefficient polynomial in x1: numpy's evaluation and the generated C's round
    # differently, and the polynomial's cancellation amplifies that to ~1e-9
    assert np.abs(ic - ref).max() <= 1e-8 * np.abs(ref).max(), float(np.abs(ic - ref).max())
    # the spanwise momentum (exact trigonometric values) agrees to rounding
    assert np.abs(ic[3] - ref[3]).max() <= 1e-15
    assert json.load(open(tmp_path / "plan.json"))["n"] == [32, 24, 8]


def test_writer_refuses_kernels_outside_the_lowered_families():
    """Extra equation classes add kernels to the time loop; lowering without them would change the
    solution, so the writer refuses every kernel it does not lower.  The WENO filter with the constant
    dissipation sensor is lowered; its Ducros variant adds a shock-sensor kernel and is refused."""
    from opensbli_gb300.writer import GB300Writer
    for case in ("tgv_central", "tgv_weno", "tgsym_central", "katzer_teno", "katzer_adaptive", "katzer_carpenter",
                 "tgv_filter", "tgv_teno_adaptive", "sbli3d_teno", "transitional_sbli", "channel_teno",
                 "shock_reflection", "sod", "shu_osher", "euler_wave", "viscous_shock_tube", "laminar_channel"):
        GB300Writer._check_kernel_families(golden_plan(case).kernels)
    assert "User kernel: Non-linear filter application" in golden_plan("tgv_filter").kernels
    names = golden_plan("tgv_filter").kernels + ["User kernel: Shock sensor"]
    with pytest.raises(NotImplementedError, match="Shock sensor"):
        GB300Writer._check_kernel_families(names)
    with pytest.raises(NotImplementedError, match="User defined thing"):
        GB300Writer._check_kernel_families(golden_plan("tgv_central").kernels + ["User defined thing"])


def test_carpenter_faces_lower_to_their_closure():
    """Faces constructed without scheme= take the reference's default Carpenter closure; the writer
    reads each face's closure from the derivative kernels' boundary conditions."""
    g = golden_plan("katzer_carpenter")
    assert g.closure == (("reduced_access", "carpenter"), ("carpenter", "reduced_access"))
    assert golden_plan("katzer_teno").closure == (("reduced_access", "reduced_access"),) * 2


def test_cfl_dt_tgv_weno():
    p = tgv_plan(256, conv="weno5js", Minf=1.25)
    dt = tgv_cfl_dt(p)
    assert 1e-3 < dt < 1e-2


# Every script the writer lowers; the default CPU run re-lowers one of each block kind (the reference
# generator takes ~15 s per script), OSB_ALL_SCRIPTS=1 all of them.  The golden plans of the others
# are still checked against the plan constructors above.
ALL_SCRIPTS = ["tgv_central", "tgv_weno", "tgv_wenoz", "tgv_teno", "tgv_teno6", "tgsym_central", "katzer_teno",
               "katzer_adaptive", "katzer_carpenter", "tgv_filter", "katzer_weno", "katzer_wenoz", "katzer_teno6",
               "tgv_teno_adaptive", "sbli3d_teno", "transitional_sbli", "channel_teno", "shock_reflection", "sod",
               "shu_osher", "euler_wave", "viscous_shock_tube", "laminar_channel"]
SCRIPTS = ALL_SCRIPTS if os.environ.get("OSB_ALL_SCRIPTS") == "1" else \
    ["tgv_weno", "katzer_adaptive", "channel_teno", "shock_reflection", "sod", "laminar_channel"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "opensbli")), reason="reference tree not present")
@pytest.mark.parametrize("case", SCRIPTS)
def test_writer_lowers_reference_script(case, tmp_path):
    r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", case, "--out",
                        str(tmp_path), "--ref", REF], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    p = Plan.from_json(open(tmp_path / "plan.json").read())
    g = golden_plan(case)
    assert p.replace(kernels=[]) == g.replace(kernels=[])
    assert sorted(p.kernels) == sorted(g.kernels)
    # the script's HDF5 output requests, as GB300Writer.run carries them out
    import json
    io = json.load(open(tmp_path / "io.json"))
    writes = [r for r in io if r["kind"] == "write"]
    assert len(writes) == 1 and writes[0]["at_end"]
    conserved = ["rho_B0", "rhou0_B0"] + (["rhou1_B0"] if p.ndim >= 2 else []) + \
        (["rhou2_B0"] if p.ndim == 3 else []) + ["rhoE_B0"]
    assert writes[0]["arrays"][:len(conserved)] == conserved
    if case == "katzer_adaptive":
        assert writes[0]["arrays"][len(conserved):] == ["x0_B0", "x1_B0", "D11_B0", "TENO_B0"]
    ic = np.load(tmp_path / "ic.npy")
    if p.ndim == 1:
        assert ic.shape == (3, p.n[0] + 8)
    elif p.ndim == 2:
        assert ic.shape == (4, p.n[1] + 8, p.n[0] + 8)  # 4-point halo: the initialisation kernel fills halos
    else:
        assert ic.shape == (5,) + tuple(reversed(p.n))
    assert np.isfinite(ic).all()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "opensbli")), reason="reference tree not present")
@pytest.mark.parametrize("variant,what", [("bulk", "Viscous residual"), ("heat", "Viscous residual")])
def test_writer_refuses_other_physics_with_the_same_kernel_names(variant, what, tmp_path):
    """A script whose stress tensor carries a bulk-viscosity term, or whose heat-flux coefficient
    differs, generates the same kernel names as the Taylor-Green WENO case; the writer evaluates the
    equations behind them and refuses (opensbli_gb300/physics_check.py)."""
    env = dict(os.environ, OSB_PHYSICS_VARIANT=variant)
    r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case",
                        "tgv_weno_modified", "--out", str(tmp_path), "--ref", REF], capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode != 0
    assert "NotImplementedError" in r.stderr and what in r.stderr, r.stderr[-2000:]


def test_physics_check_catches_a_changed_constituent_relation():
    """Unit check of the constituent-relation comparison on a hand-made kernel list."""
    import sympy
    from opensbli_gb300 import physics_check as P

    class DS(sympy.Symbol):  # stands in for the reference's DataSet (class name is what is checked)
        pass
    DS.__name__ = "DataSet"

    class K:  # stands in for the reference's Kernel
        def __init__(self, name, eqs):
            self.computation_name, self.equations = name, eqs
    K.__name__ = "Kernel"

    def ds(name):
        d = DS(name + "_B0")
        d.base, d.indices = name + "_B0", (0, 0, 0)
        return d
    rho, m0, m1, m2, E = (ds(n) for n in ("rho", "rhou0", "rhou1", "rhou2", "rhoE"))
    g = 1.4
    good = [K("CRu%d" % c, [sympy.Eq(ds("u%d" % c), m / rho)]) for c, m in enumerate((m0, m1, m2))]
    p_ok = K("CRp", [sympy.Eq(ds("p"), (g - 1) * (E - (m0 ** 2 + m1 ** 2 + m2 ** 2) / (2 * rho)))])
    p_bad = K("CRp", [sympy.Eq(ds("p"), (g - 1) * (E - (m0 ** 2 + m1 ** 2) / (2 * rho)))])
    P.PhysicsCheck(good + [p_ok], 3, viscous=False).check_constituent_relations()
    with pytest.raises(NotImplementedError, match="constituent relation for p"):
        P.PhysicsCheck(good + [p_bad], 3, viscous=False).check_constituent_relations()
