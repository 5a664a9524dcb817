"""GB300Writer: the backend seam beside OpenSBLI's OPSC writer.

A problem script builds its algorithm exactly as for OPS:

    alg = TraditionalAlgorithmRK(block)
    SimulationDataType.set_datatype(Double)
    OPSC(alg)                                   # reference backend: writes C for OPS
    GB300Writer(alg, precision='fp64')          # this backend: lowers alg to a Plan

The OPSC writer (code_generation/opsc.py:250-282) walks alg.prg and prints every Kernel as an
ops_par_loop.  GB300Writer walks the same tree (opsc.py:595-609 traversal) and recognises the
kernel families of the hot path -- constituent relations, Central skew-symmetric convective terms,
LLFWeno reconstructions, viscous terms, the RK stage kernels and the boundary exchanges -- and
lowers them to one Plan that selects the fused GB300 kernels.  Anything it does not recognise
raises NotImplementedError: there is no generic fallback and no CPU path.

Constants get their values the way the reference's scripts give them: through
substitute_simulation_parameters(constants, values) (utilities/helperfunctions.py:130-149), here a
method of the writer taking the same two lists.
"""
import math
import re

import numpy as np

from . import physics_check
from .plan import Plan

_C_NAMES = {"M_PI": math.pi, "pi": math.pi, "ceil": math.ceil, "floor": math.floor, "sqrt": math.sqrt,
            "sin": math.sin, "cos": math.cos, "exp": math.exp, "log": math.log, "pow": math.pow, "fabs": abs}


def _eval_c_expr(expr, env):
    """Evaluate the small C expressions problem scripts pass as values ('2*M_PI/block0np0')."""
    if not re.fullmatch(r"[0-9A-Za-z_+\-*/(). eE]+", expr):
        raise ValueError("unsupported value expression %r" % expr)
    names = dict(_C_NAMES)
    names.update(env)
    return eval(expr, {"__builtins__": {}}, names)


def _walk(component, out):
    for c in getattr(component, "components", []) or []:
        out.append(c)
        _walk(c, out)
    return out


class GB300Writer:
    """Lower an OpenSBLI TraditionalAlgorithmRK to a Plan for libosbli_gb300.

    :arg algorithm: the TraditionalAlgorithmRK of the problem script (same positional argument as
        OPSC).
    :arg str precision: 'fp64' (the reference's Double) or 'mixed' (FP32 state and flux arithmetic,
        FP64 RK accumulator).
    """

    def __init__(self, algorithm, precision="fp64", use_graphs=True):
        self.algorithm = algorithm
        if getattr(algorithm, "MultiBlock", False) or len(algorithm.block_descriptions) != 1:
            raise NotImplementedError("GB300Writer lowers single-block algorithms")
        self.block = algorithm.block_descriptions[0]
        self.components = _walk(algorithm.prg, [])
        self.kernel_names = [getattr(c, "computation_name", None) for c in self.components
                             if type(c).__name__ == "Kernel"]
        self.values = {}
        self.plan = self._lower(precision, use_graphs)
        self.ic_kernel = self._find_kernel("Grid_based_initialisation")

    # ------------------------------------------------------------------ recognition
    def _find_kernel(self, prefix):
        for c in self.components:
            if type(c).__name__ == "Kernel" and (c.computation_name or "").startswith(prefix):
                return c
        return None

    def _kernels(self, prefix):
        return [c for c in self.components
                if type(c).__name__ == "Kernel" and (c.computation_name or "").startswith(prefix)]

    @staticmethod
    def _max_offset(kernels):
        from sympy import preorder_traversal
        m = 0
        for k in kernels:
            for e in k.equations:
                for a in preorder_traversal(e.rhs):
                    if type(a).__name__ == "DataSet":
                        m = max([m] + [abs(int(i)) for i in a.indices])
        return m

    @staticmethod
    def _lhs_names(kernel):
        return {str(e.lhs) for e in kernel.equations}

    def _lower(self, precision, use_graphs):
        """Recognise the kernel families in alg.prg and build the Plan (all information comes from the
        algorithm tree, as for the OPSC writer)."""
        names = [n or "" for n in self.kernel_names]
        self._check_kernel_families(names)
        ndim = self.block.ndim
        if ndim in (1, 2) or (ndim == 3 and any(n.startswith("IsothermalWall boundary") for n in names)):
            return self._lower_2d(precision, use_graphs)
        if ndim != 3:
            raise NotImplementedError("GB300Writer lowers 2D and 3D blocks (got ndim=%d)" % ndim)
        skew = self._kernels("Convective terms group")
        weno = self._kernels("LLFWeno_reconstruction_")
        teno = self._kernels("LLFTeno_reconstruction_")
        visc = self._kernels("Viscous")
        if [bool(skew), bool(weno), bool(teno)].count(True) != 1:
            raise NotImplementedError("expected exactly one convective discretisation (Central skew, LLFWeno or "
                                      "LLFTeno)")
        if teno:
            # LLFTeno(5) with a fixed or Ducros-adapted cut-off (teno.py:407-465); LLFTeno(6) adds a
            # fourth candidate stencil (delta_3, teno.py:94-105)
            conv = "teno6" if all("delta_3" in self._lhs_names(k) for k in teno) else "teno5"
            if len(teno) != 3:
                raise NotImplementedError("one LLFTeno reconstruction kernel per direction expected")
            for k in teno:
                lhs = self._lhs_names(k)
                if not {"delta_0", "delta_1", "delta_2", "inv_omega_sum"} <= lhs:
                    raise NotImplementedError("TENO5 with a cut-off expected in %s" % k.computation_name)
                if self._max_offset([k]) != 3:
                    raise NotImplementedError("5th-order stencil expected in %s" % k.computation_name)
                avg = [e for e in k.equations if str(e.lhs).endswith("_rho") and str(e.lhs).startswith("AVG_")]
                if not avg or "sqrt" not in str(avg[0].rhs):
                    raise NotImplementedError("Roe averaging expected in %s" % k.computation_name)
            if not self._kernels("LLFTeno Residual"):
                raise NotImplementedError("LLFTeno residual kernel missing")
        elif skew:
            conv = "central_skew"
            if len(skew) != 3 or self._max_offset(self._kernels("Convective CD")) != 2:
                raise NotImplementedError("Central(4) skew-symmetric convective terms expected")
        else:
            conv = None
            if len(weno) != 3:
                raise NotImplementedError("one LLFWeno reconstruction kernel per direction expected")
            for k in weno:
                lhs = self._lhs_names(k)
                if not {"beta_0", "beta_1", "beta_2", "alpha_0", "omega_0", "inv_alpha_sum"} <= lhs:
                    raise NotImplementedError("WENO5 reconstruction expected in %s" % k.computation_name)
                # WenoZ's alphas carry the global indicator |beta_0 - beta_2| (weno.py:283-331)
                alpha0 = [e for e in k.equations if str(e.lhs) == "alpha_0"]
                kconv = "weno5z" if alpha0 and "Abs(" in str(alpha0[0].rhs) else "weno5js"
                if conv not in (None, kconv):
                    raise NotImplementedError("mixed WENO formulations across directions")
                conv = kconv
                if self._max_offset([k]) != 3:
                    raise NotImplementedError("5th-order stencil expected in %s" % k.computation_name)
                avg = [e for e in k.equations if str(e.lhs).endswith("_rho") and str(e.lhs).startswith("AVG_")]
                if not avg or "sqrt" not in str(avg[0].rhs):
                    raise NotImplementedError("Roe averaging expected in %s" % k.computation_name)
            if not self._kernels("LLFWeno Residual"):
                raise NotImplementedError("LLFWeno residual kernel missing")
        if visc and self._max_offset(visc) != 2:
            raise NotImplementedError("Central(4) viscous terms expected")
        # constituent relations: u_i, p, T (and a for WENO), constant viscosity
        base = {re.sub(r"_B0$", "", n) for n in names if n.startswith("CR")}
        need = {"CRu0", "CRu1", "CRu2", "CRp"} | ({"CRT"} if visc else set()) | ({"CRa"} if weno or teno else set())
        if not need <= base or base - need - {"CRT", "CRa"}:
            raise NotImplementedError("unsupported constituent relations: %s" % sorted(base))
        # RK3 coefficients from the stage kernels (rk_sbli.py:102-124)
        from sympy import preorder_traversal
        coeff = {}
        for kname in ("Sub stage advancement", "Temporal solution advancement"):
            ks = self._kernels(kname)
            if len(ks) != 1:
                raise NotImplementedError("RungeKutta(3) stage kernels expected")
            for e in ks[0].equations:
                for a in preorder_traversal(e.rhs):
                    if type(a).__name__ == "ConstantIndexed":
                        coeff[str(a.base)] = tuple(float(v) for v in a.value)
        if set(coeff) != {"rkold", "rknew"} or len(coeff["rkold"]) != 3:
            raise NotImplementedError("2-register RK3 coefficients rkold/rknew expected")
        # boundary conditions: periodic exchanges or symmetry boundary kernels, per axis and side
        bcs = [[None, None] for _ in range(3)]
        for c in self.components:
            if type(c).__name__ == "ExchangeSelf":
                bcs[c.direction][0 if c.side == "left" else 1] = "periodic"
        for d in range(3):
            for side in range(2):
                if self._kernels("Symmetry boundary dir%d side%d" % (d, side)):
                    bcs[d][side] = "symmetry"
        other_bc = [n for n in names if "boundary dir" in n and not n.startswith("Symmetry")]
        if other_bc or any(b is None for pair in bcs for b in pair):
            raise NotImplementedError("unsupported boundary conditions: %s" % (other_bc or bcs))
        filt, fc = self._weno_filter()
        adaptive = self._adaptive_teno(teno) if teno else None
        if adaptive is None and self._kernels("ConstituentRelations CD"):
            raise NotImplementedError("sensor derivative kernels without the adaptive TENO cut-off")
        # the equations behind the recognised kernels must be the physics the fused kernels implement
        physics_check.check_algorithm(self.components, 3, viscous=bool(visc), skew=conv == "central_skew")
        return Plan(ndim=3, conv=conv, visc="const" if visc else "none", rk="rk3", precision=precision,
                    bc=tuple(tuple(p) for p in bcs), rk_a=coeff["rkold"], rk_b=coeff["rknew"],
                    weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
                    use_graphs=use_graphs, ic="host", kernels=[n for n in names if n], filter=filt,
                    filter_control=fc, teno_adaptive=adaptive is not None,
                    sensor_eps=adaptive if adaptive is not None else Plan.sensor_eps)

    def _weno_filter(self):
        """Recognise the WENO5 non-linear filter (filters/WENO_filter.py:15-339) in the time loop: its
        constituent relations, one reconstruction kernel per direction (LLFWeno(5, 'JS') with the simple
        average, the weight sensor rj and the central subtraction, shock_capturing.py:399-442) and the
        application kernel q += dt * shock_filter_control * Wall * kappa * R.  Returns (filter kind,
        shock_filter_control).  Only the 'Constant' dissipation sensor (kappa = 1) is lowered; the
        Ducros sensor's kernels are refused."""
        recon = self._kernels("User kernel: WENO reconstruction direction")
        app = self._kernels("User kernel: Non-linear filter application")
        cr = self._kernels("User kernel: Constituent Relations evaluation")
        if not recon and not app and not cr:
            return "none", 1.0
        if len(recon) != 3 or len(app) != 1 or len(cr) != 1:
            raise NotImplementedError("WENO filter: one reconstruction kernel per direction, one constituent-"
                                      "relation and one application kernel expected")
        for k in recon:
            lhs = self._lhs_names(k)
            if not {"beta_0", "alpha_0", "omega_0", "rj0", "Recon_0"} <= lhs:
                raise NotImplementedError("WENO filter: WENO5 reconstruction with the weight sensor expected in %s"
                                          % k.computation_name)
            if self._max_offset([k]) != 3:
                raise NotImplementedError("WENO filter: 5th-order stencil expected in %s" % k.computation_name)
            avg = [e for e in k.equations if str(e.lhs).startswith("AVG_") and str(e.lhs).endswith("_rho")]
            if not avg or "sqrt" in str(avg[0].rhs):
                raise NotImplementedError("WENO filter: the simple average expected in %s" % k.computation_name)
            alpha0 = [e for e in k.equations if str(e.lhs) == "alpha_0"]
            if not alpha0 or "Abs(" in str(alpha0[0].rhs):
                raise NotImplementedError("WENO filter: WENO-JS weights expected in %s" % k.computation_name)
        fc, kappa = None, False
        from sympy import preorder_traversal
        for e in app[0].equations:
            for a in preorder_traversal(e.rhs):
                if type(a).__name__ == "ConstantObject" and str(a) == "shock_filter_control":
                    fc = float(a.value)
                elif "kappa" in str(a) and type(a).__name__ in ("DataSet", "GridVariable"):
                    kappa = True
            if str(e.lhs) == "Wall" and str(e.rhs) != "1":
                raise NotImplementedError("WENO filter next to wall faces is not lowered (3D periodic/symmetry "
                                          "blocks only)")
        if kappa or self._kernels("User kernel: Shock sensor"):
            raise NotImplementedError("WENO filter with the Ducros dissipation sensor is not lowered "
                                      "(dissipation_sensor='Constant' is)")
        if fc is None:
            raise NotImplementedError("WENO filter: shock_filter_control not found in the application kernel")
        return "weno5_constant", fc

    # The kernel families this writer lowers (by the computation names the reference gives them);
    # anything else in the time loop (filters, other equation classes, user kernels) would be
    # dropped silently, so it is refused.
    _FAMILIES = re.compile(
        r"^(CR\w+|ConstituentRelations (evaluation|CD )|Convective (CD |residual|terms group|terms$)|Derivative evaluation CD |"
        r"LLF(Weno|Teno)(_reconstruction_\d+_direction| Residual)|MetricsEquation|Viscous|Grid_based_initialisation|"
        r"Save equations|Sub stage advancement|Temporal solution advancement|\w+ boundary dir\d side\d|"
        r"User kernel: (Constituent Relations evaluation|WENO reconstruction direction \d|Non-linear filter application))")

    @classmethod
    def _check_kernel_families(cls, names):
        other = sorted({n for n in names if n and not cls._FAMILIES.match(n)})
        if other:
            raise NotImplementedError("kernels outside the lowered families (filters, user-defined or other "
                                      "equation classes are not lowered): %s" % other)

    def _rk_coefficients(self, names_expected):
        from sympy import preorder_traversal
        coeff = {}
        for kname in names_expected:
            ks = self._kernels(kname)
            if len(ks) != 1:
                raise NotImplementedError("RK stage kernel %r expected" % kname)
            for e in ks[0].equations:
                for a in preorder_traversal(e.rhs):
                    if type(a).__name__ == "ConstantIndexed":
                        coeff[str(a.base)] = tuple(float(v) for v in a.value)
        return coeff

    def _lower_2d(self, precision, use_graphs):
        """2D wall-bounded blocks (apps/katzer_SBLI/katzer_SBLI.py with a fixed TENO cut-off): metrics
        stretched in x1, LLFTeno(5) or LLFWeno(5), Central(4) viscous terms with Sutherland viscosity,
        RungeKuttaLS(3), inlet/extrapolation faces in x0, isothermal wall/Dirichlet faces in x1; and
        the same block in 3D with a periodic x2 axis (apps/transitional_SBLI/transitional_SBLI.py's
        block without its body force)."""
        import sympy
        names = [n or "" for n in self.kernel_names]
        nd = self.block.ndim
        if any(n.startswith("User kernel:") for n in names):
            raise NotImplementedError("the WENO filter is lowered on 3D blocks only")
        teno = self._kernels("LLFTeno_reconstruction_")
        weno = self._kernels("LLFWeno_reconstruction_")
        if nd == 2 and not teno and not weno and self._kernels("Convective terms"):
            return self._lower_skew2d(precision, use_graphs, names)
        if bool(teno) == bool(weno) or len(teno or weno) != nd:
            raise NotImplementedError("wall-bounded blocks: one LLFTeno or LLFWeno reconstruction per direction "
                                      "expected")
        conv = None
        for k in teno:
            lhs = self._lhs_names(k)
            if not {"delta_0", "delta_1", "delta_2", "inv_omega_sum"} <= lhs:
                raise NotImplementedError("TENO5 with a cut-off expected in %s" % k.computation_name)
            kconv = "teno6" if "delta_3" in lhs else "teno5"  # LLFTeno(6) adds a fourth candidate
            if conv not in (None, kconv):
                raise NotImplementedError("mixed TENO orders across directions")
            conv = kconv
        for k in weno:
            lhs = self._lhs_names(k)
            if not {"beta_0", "beta_1", "beta_2", "alpha_0", "omega_0", "inv_alpha_sum"} <= lhs:
                raise NotImplementedError("WENO5 reconstruction expected in %s" % k.computation_name)
            # WenoZ's alphas carry the global indicator |beta_0 - beta_2| (weno.py:283-331)
            alpha0 = [e for e in k.equations if str(e.lhs) == "alpha_0"]
            kconv = "weno5z" if alpha0 and "Abs(" in str(alpha0[0].rhs) else "weno5js"
            if conv not in (None, kconv):
                raise NotImplementedError("mixed WENO formulations across directions")
            conv = kconv
        adaptive = self._adaptive_teno(teno) if teno else None
        if adaptive is not None and conv not in (("teno5",) if nd == 2 else ("teno5", "teno6")):
            raise NotImplementedError("the adaptive cut-off is lowered for TENO5 (2D) and TENO5/TENO6 (3D) blocks")
        if self._max_offset(teno or weno) != 3:
            raise NotImplementedError("5th-order reconstruction stencil expected")
        averaging = self._averaging(teno or weno)
        # a 2D Euler block (apps/inviscid_shock_reflection/inviscid_shock.py): no viscous kernels, no metric
        euler = nd <= 2 and not any(n.startswith(("CRmu", "CRT", "Viscous")) for n in names)
        if euler:
            if self._kernels("MetricsEquation") or self._kernels("Metric boundary"):
                raise NotImplementedError("Euler blocks: Cartesian grids only")
            return self._lower_euler2d(precision, use_graphs, conv, averaging, names)
        if nd == 1:
            raise NotImplementedError("1D blocks: the Euler equations")
        if nd == 2 and not self._kernels("MetricsEquation") and not self._kernels("Metric boundary"):
            return self._lower_viscous2d_cartesian(precision, use_graphs, conv, averaging, names)
        if not self._kernels("MetricsEquation") or not self._kernels("Metric boundary"):
            raise NotImplementedError("2D blocks: metric terms expected")
        if not any(n.startswith("CRmu") for n in names):
            raise NotImplementedError("wall-bounded blocks: a viscosity relation (CRmu) expected")
        visc_exp = self._power_law_viscosity()
        if visc_exp is not None and nd != 3:
            raise NotImplementedError("2D blocks: Sutherland viscosity")
        if averaging != "roe":
            raise NotImplementedError("wall-bounded blocks: the Roe average expected")
        coeff = self._rk_coefficients(["Temporal solution advancement"])
        if set(coeff) != {"rkA", "rkB"}:
            raise NotImplementedError("RungeKuttaLS(3) coefficients rkA/rkB expected")
        faces = {
            "InletPressureExtrapolate boundary dir0 side0": ("inlet_pressure_extrapolate", 0, 0),
            "Extrapolation boundary dir0 side1": ("extrapolation", 0, 1),
            "IsothermalWall boundary dir1 side0": ("isothermal_wall", 1, 0),
            "Dirichlet boundary dir1 side1": ("dirichlet", 1, 1),
            "IsothermalWall boundary dir1 side1": ("isothermal_wall", 1, 1),
        }
        bcs = [[None, None], [None, None]]
        for kname, (kind, d, side) in faces.items():
            if self._kernels(kname):
                if bcs[d][side] is not None:
                    raise NotImplementedError("two boundary conditions on face dir%d side%d" % (d, side))
                bcs[d][side] = kind
        # a periodic x0 (the channel, apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py): the
        # exchanges of both sides and no boundary kernel on that axis
        per0 = {c.side for c in self.components if type(c).__name__ == "ExchangeSelf" and c.direction == 0}
        if nd == 3 and per0 == {"left", "right"} and bcs[0] == [None, None]:
            bcs[0] = ["periodic", "periodic"]
        known = ([["inlet_pressure_extrapolate", "extrapolation"], ["isothermal_wall", "dirichlet"]],
                 [["periodic", "periodic"], ["isothermal_wall", "isothermal_wall"]])
        if bcs not in known or (bcs == known[1] and nd != 3):
            found = sorted(n for n in names if "boundary dir" in n)
            raise NotImplementedError("wall-bounded boundary conditions: %s" % found)
        channel = bcs == known[1]
        if channel and visc_exp is None:
            raise NotImplementedError("channel blocks: the power-law viscosity expected")
        if nd == 3:
            # x2 periodic: the exchanges of both sides and no boundary kernel on that axis
            per = {c.side for c in self.components if type(c).__name__ == "ExchangeSelf" and c.direction == 2}
            other = [n for n in names if "boundary dir" in n and n not in faces and not n.startswith("Metric boundary")]
            if per != {"left", "right"} or other:
                raise NotImplementedError("3D wall-bounded blocks: periodic x2 expected (found %s)" % (other or per))
        closure = self._closures_2d(periodic0=channel)
        # the Dirichlet face: rho, rhou0, rhou1 (, rhou2), rhoE = Piecewise((hi, x0 > xs), (lo, True)); on 3D
        # blocks rhoE may instead be a constant plus the point's spanwise kinetic energy
        # rhou2^2/(2 rho) with rhou2 left as it is (apps/transitional_SBLI/transitional_SBLI.py:110-116)
        dk = self._kernels("Dirichlet boundary dir1 side1")
        lo, hi, xs, ke = {}, {}, None, False

        def value(v, name):
            nonlocal ke
            ds = [a for a in sympy.preorder_traversal(v) if type(a).__name__ == "DataSet"]
            if not ds:
                return float(v)
            names = {re.sub(r"_B0$", "", str(a.base)) for a in ds}
            if nd != 3 or name != "rhoE" or names != {"rho", "rhou2"} or any(int(i) != 0 for a in ds for i in a.indices):
                raise NotImplementedError("Dirichlet face: %s = %s is not lowered" % (name, v))
            r2, rh = sympy.symbols("_osb_r2 _osb_rho")
            f = v.xreplace({a: (r2 if str(a.base).startswith("rhou2") else rh) for a in ds})
            c = float(f.subs({r2: 0, rh: 1}))
            for tv, rv in ((0.37, 1.3), (-1.1, 0.6)):
                if abs(float(f.subs({r2: tv, rh: rv})) - (c + 0.5 * tv * tv / rv)) > 1e-12:
                    raise NotImplementedError("Dirichlet face: rhoE = %s is not const + rhou2^2/(2 rho)" % v)
            ke = True
            return c

        for e in (dk[0].equations if dk else []):
            name = re.sub(r"_B0$", "", str(getattr(e.lhs, "base", e.lhs)))
            rhs = e.rhs
            if isinstance(rhs, sympy.Piecewise) and len(rhs.args) == 2:
                (vhi, cond), (vlo, _) = rhs.args
                if not isinstance(cond, sympy.core.relational.StrictGreaterThan):
                    raise NotImplementedError("Dirichlet face: state switched by x0 > value expected")
                xs = float(cond.rhs)
                hi[name], lo[name] = value(vhi, name), value(vlo, name)
            elif name in ("rho", "rhou0", "rhou1", "rhou2", "rhoE"):
                hi[name] = lo[name] = value(rhs, name)
        order = ["rho", "rhou0", "rhou1"] + (["rhou2"] if nd == 3 else []) + ["rhoE"]
        if ke:
            if "rhou2" in lo:
                raise NotImplementedError("Dirichlet face: rhou2 set with rhoE carrying its kinetic energy")
            lo["rhou2"] = hi["rhou2"] = 0.0  # kept at the face, not set
        if dk and any(v not in lo for v in order):
            raise NotImplementedError("Dirichlet face must set %s" % ", ".join(order))
        bf = self._body_force() if nd == 3 else None
        forcing = self._forcing(teno or weno) if nd == 3 else None
        physics_check.check_algorithm(self.components, nd, viscous=True, sutherland=True, metric=True,
                                      body_force=bf is not None, visc_exp=visc_exp, forcing=forcing is not None)
        extra = {}
        if channel:  # the coordinate line comes from the script's grid equations (initial_fields)
            extra = dict(visc_exp=visc_exp, forcing=forcing, x1_grid="tanh")
        else:
            extra = dict(dirichlet_lo=tuple(lo[v] for v in order), dirichlet_hi=tuple(hi[v] for v in order),
                         dirichlet_x_switch=xs if xs is not None else 1e300)
        return Plan(ndim=nd, n=(64, 32, 1) if nd == 2 else (64, 32, 16), delta=(1.0, 1.0, 1.0), conv=conv,
                    weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
                    visc="power" if channel else "sutherland", rk="ls_rk3", precision=precision,
                    bc=(tuple(bcs[0]), tuple(bcs[1]), ("periodic", "periodic")),
                    rk_a=coeff["rkA"], rk_b=coeff["rkB"], use_graphs=use_graphs, ic="host",
                    name=("channel" if channel else "wall3d") if nd == 3 else Plan.name,
                    kernels=[n for n in names if n], dirichlet_ke=ke, body_force=bf, **extra,
                    teno_adaptive=adaptive is not None,
                    sensor_eps=adaptive if adaptive is not None else Plan.sensor_eps, closure=closure)

    _BF_CONSTS = ("A", "xF", "yF", "bta", "omega")

    def _averaging(self, reconstruction):
        """The average the characteristic system is built from, read from the reconstruction kernels'
        AVG_*_rho equations: "roe" (sqrt(rho_l rho_r), averaging.py:62-114) or "simple" ((rho_l +
        rho_r)/2, averaging.py:31-59); both checked numerically."""
        import sympy
        kinds = set()
        for k in reconstruction:
            avg = [e for e in k.equations if re.match(r"AVG_\d+_rho$", str(e.lhs))]
            if len(avg) != 1:
                raise NotImplementedError("averaged density expected in %s" % k.computation_name)
            ds = [a for a in sympy.preorder_traversal(avg[0].rhs) if type(a).__name__ == "DataSet"]
            if len(ds) != 2 or {str(a.base) for a in ds} != {"rho_B0"}:
                raise NotImplementedError("averaged density of %s reads %s" % (k.computation_name, ds))
            val = float(avg[0].rhs.xreplace({ds[0]: sympy.Float(1.3), ds[1]: sympy.Float(0.7)}))
            if abs(val - 1.0) < 1e-14:
                kinds.add("simple")
            elif abs(val - (1.3 * 0.7) ** 0.5) < 1e-14:
                kinds.add("roe")
            else:
                raise NotImplementedError("average of %s not recognised" % k.computation_name)
        if len(kinds) != 1:
            raise NotImplementedError("one average for every direction expected")
        return kinds.pop()

    def _face_states(self, kname, consts, nd=2):
        """Evaluate a Dirichlet face kernel (dirichlet.py:6-41) as the generated code does, in equation
        order with its locals, the constants in `consts`, and x0 a free variable.  Returns (lo, hi, xs):
        the states (rho, rhou0, rhou1, rhoE) where x0 <= xs and where x0 > xs (xs = 1e300: one state)."""
        import math
        import sympy
        ks = self._kernels(kname)  # the face is applied before the loop and after every stage
        if not ks or any(k.equations != ks[0].equations for k in ks):
            raise NotImplementedError("one %s kernel expected" % kname)
        x = sympy.Symbol("_osb_x0")
        env, out, thresholds = {}, {}, set()
        for e in ks[0].equations:
            reps = {}
            it = sympy.preorder_traversal(e.rhs)
            for a in it:
                t = type(a).__name__
                if t == "DataSet":
                    it.skip()  # not its shape constants
                    if str(a.base) != "x0_B0" or any(int(i) != 0 for i in a.indices):
                        raise NotImplementedError("Dirichlet face reads %s" % a)
                    reps[a] = x
                elif t == "ConstantObject":
                    if str(a) in consts:  # others (a grid spacing of an unused local) stay symbols
                        reps[a] = sympy.Float(consts[str(a)], 30)
                elif t == "GridVariable" or (isinstance(a, sympy.Symbol) and t == "Symbol"):
                    # the kernel's locals, else a constant the generated code reads by name (a script
                    # that parses "gama" without declaring it a ConstantObject); the generated code
                    # initialises every local to 0.0, so one read before it is set reads 0
                    # (shu_osher.py's outlet face reads u0 so)
                    if str(a) in env:
                        reps[a] = env[str(a)]
                    elif str(a) in consts and t == "Symbol":
                        reps[a] = sympy.Float(consts[str(a)], 30)
                    else:
                        reps[a] = sympy.Float(0)
            v = e.rhs.xreplace(reps)
            for r in sympy.preorder_traversal(v):
                if isinstance(r, sympy.core.relational.Relational) and r.free_symbols == {x}:
                    sol = sympy.solve(sympy.Eq(r.lhs, r.rhs), x)
                    thresholds.update(float(t) for t in sol)
            if type(e.lhs).__name__ == "GridVariable":
                env[str(e.lhs)] = v
            else:
                out[re.sub(r"_B0$", "", str(getattr(e.lhs, "base", e.lhs)))] = v
        order = ["rho", "rhou0", "rhou1", "rhoE"] if nd == 2 else ["rho", "rhou0", "rhoE"]
        if set(out) != set(order):
            raise NotImplementedError("%s sets %s" % (kname, sorted(out)))
        for n_ in order:
            if out[n_].free_symbols - {x}:
                raise NotImplementedError("%s: %s depends on %s" % (kname, n_, out[n_].free_symbols - {x}))

        def at(xv):
            return tuple(float(out[n].subs(x, xv)) for n in order)
        if not thresholds:
            st = at(0.0)
            return st, st, 1e300
        if len(thresholds) != 1:
            raise NotImplementedError("%s: one switch location expected" % kname)
        c = thresholds.pop()
        lo, hi, mid = at(c - 1.0), at(c + 1.0), at(c)
        if mid not in (lo, hi) or any(at(xv) != lo for xv in (c - 5.0, c - 100.0)) or \
                any(at(xv) != hi for xv in (c + 5.0, c + 100.0)):
            raise NotImplementedError("%s: a state switched at one x0 location expected" % kname)
        # the kernels compare x0 > xs: a switch that includes c itself moves xs just below it
        return lo, hi, (c if mid == lo else math.nextafter(c, -math.inf))

    def _lower_skew2d(self, precision, use_graphs, names):
        """The 2D laminar channel (apps/channel_flow/laminar_2D/laminar_channel.py): central skew-symmetric
        convective terms (one "Convective terms" kernel), central viscous terms with Sutherland's law on a
        Cartesian grid, the constant forcing c_j, periodic x0, isothermal walls on both x1 faces,
        RungeKuttaLS(3)."""
        import sympy
        if self._kernels("MetricsEquation") or self._kernels("Metric boundary"):
            raise NotImplementedError("2D central-skew blocks: Cartesian grids only")
        if not any(n.startswith("CRmu") for n in names) or self._power_law_viscosity() is not None:
            raise NotImplementedError("2D central-skew blocks: Sutherland viscosity expected")
        coeff = self._rk_coefficients(["Temporal solution advancement"])
        if set(coeff) != {"rkA", "rkB"}:
            raise NotImplementedError("RungeKuttaLS(3) coefficients rkA/rkB expected")
        found = {n for n in names if "boundary dir" in n}
        exch = {(c.direction, c.side) for c in self.components if type(c).__name__ == "ExchangeSelf"}
        if found != {"IsothermalWall boundary dir1 side0", "IsothermalWall boundary dir1 side1"} or \
                exch != {(0, "left"), (0, "right")}:
            raise NotImplementedError("2D central-skew block boundary conditions: %s" % sorted(found))
        forcing = {}
        for k in self._kernels("Convective terms"):
            for e in k.equations:
                for a in sympy.preorder_traversal(e.rhs):
                    if type(a).__name__ == "ConstantObject" and re.fullmatch(r"c[0-1]", str(a)):
                        forcing[int(str(a)[1])] = a
        closure = self._closures_2d(periodic0=True)
        physics_check.check_algorithm(self.components, 2, viscous=True, sutherland=True, metric=False, skew=True,
                                      forcing=bool(forcing))
        vals = [getattr(forcing.get(d), "value", None) for d in range(2)]
        return Plan(ndim=2, n=(64, 32, 1), delta=(1.0, 1.0, 1.0), conv="central_skew", visc="sutherland",
                    rk="ls_rk3", precision=precision, x1_grid="uniform",
                    bc=(("periodic", "periodic"), ("isothermal_wall", "isothermal_wall"), ("periodic", "periodic")),
                    rk_a=coeff["rkA"], rk_b=coeff["rkB"], use_graphs=use_graphs, ic="host",
                    closure=(("none", "none"), closure[1]),
                    forcing=tuple(float(v) if isinstance(v, (int, float)) else 0.0 for v in vals) if forcing else None,
                    name="channel2d", kernels=[n for n in names if n])

    def _lower_viscous2d_cartesian(self, precision, use_graphs, conv, averaging, names):
        """A Cartesian 2D Navier-Stokes block with a constant viscosity (apps/viscous_shock_tube/
        viscous_shock_tube.py): LLFTeno/LLFWeno with the Roe average, central viscous terms, RungeKuttaLS(3),
        adiabatic walls at both x0 faces and at x1 = 0, a symmetry face at the top (each face's closure
        read from the derivative kernels).  mu is the script's constant; the kernels implement mu = 1,
        which substitute_simulation_parameters checks."""
        if any(n.startswith("CRmu") for n in names):
            raise NotImplementedError("Cartesian viscous blocks: a constant viscosity expected")
        if averaging != "roe":
            raise NotImplementedError("Cartesian viscous blocks: the Roe average expected")
        coeff = self._rk_coefficients(["Temporal solution advancement"])
        if set(coeff) != {"rkA", "rkB"}:
            raise NotImplementedError("RungeKuttaLS(3) coefficients rkA/rkB expected")
        faces = {"AdiabaticWall boundary dir0 side0", "AdiabaticWall boundary dir0 side1",
                 "AdiabaticWall boundary dir1 side0", "Symmetry boundary dir1 side1"}
        found = {n for n in names if "boundary dir" in n}
        if found != faces:
            raise NotImplementedError("Cartesian viscous block boundary conditions: %s" % sorted(found))
        closure = self._closures_2d()
        physics_check.check_algorithm(self.components, 2, viscous=True, sutherland=False, metric=False)
        return Plan(ndim=2, n=(64, 32, 1), delta=(1.0, 1.0, 1.0), conv=conv,
                    weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
                    visc="const", rk="ls_rk3", precision=precision, x1_grid="uniform",
                    bc=(("adiabatic_wall", "adiabatic_wall"), ("adiabatic_wall", "symmetry"), ("periodic", "periodic")),
                    rk_a=coeff["rkA"], rk_b=coeff["rkB"], use_graphs=use_graphs, ic="host", closure=closure,
                    name="viscous2d", kernels=[n for n in names if n])

    def _lower_euler2d(self, precision, use_graphs, conv, averaging, names):
        """A 2D Euler block (apps/inviscid_shock_reflection/inviscid_shock.py): Cartesian, no viscous terms,
        LLFWeno/LLFTeno with the Roe or the simple average, RungeKuttaLS(3); a Dirichlet or inlet face at
        x0 = 0, a Dirichlet or extrapolation face at the outlet, a symmetry face at x1 = 0 and a Dirichlet
        (possibly switched at one x0) or symmetry face at the top.  The faces' states depend on the
        simulation's constants; they are evaluated again by substitute_simulation_parameters."""
        coeff = self._rk_coefficients(["Temporal solution advancement"])
        if set(coeff) == {"rkA", "rkB"}:
            rk, rk_a, rk_b = "ls_rk3", coeff["rkA"], coeff["rkB"]
        else:  # RungeKutta(3) with two registers (euler_wave.py)
            coeff = self._rk_coefficients(["Sub stage advancement", "Temporal solution advancement"])
            if set(coeff) != {"rkold", "rknew"} or len(coeff["rkold"]) != 3:
                raise NotImplementedError("RungeKuttaLS(3) or RungeKutta(3) coefficients expected")
            rk, rk_a, rk_b = "rk3", coeff["rkold"], coeff["rknew"]
        faces = {
            "InletPressureExtrapolate boundary dir0 side0": ("inlet_pressure_extrapolate", 0, 0),
            "Dirichlet boundary dir0 side0": ("dirichlet", 0, 0),
            "Extrapolation boundary dir0 side1": ("extrapolation", 0, 1),
            "Dirichlet boundary dir0 side1": ("dirichlet", 0, 1),
            "Symmetry boundary dir1 side0": ("symmetry", 1, 0),
            "Dirichlet boundary dir1 side1": ("dirichlet", 1, 1),
            "Symmetry boundary dir1 side1": ("symmetry", 1, 1),
        }
        nd = self.block.ndim
        bcs = [[None, None], [None, None]]
        for kname, (kind, d, side) in faces.items():
            if self._kernels(kname):
                if bcs[d][side] is not None:
                    raise NotImplementedError("two boundary conditions on face dir%d side%d" % (d, side))
                bcs[d][side] = kind
        other = sorted(n for n in names if "boundary dir" in n and n not in faces)
        exch = {(c.direction, c.side) for c in self.components if type(c).__name__ == "ExchangeSelf"}
        if nd == 2 and bcs == [[None, None], [None, None]] and not other and \
                exch == {(d, side) for d in range(2) for side in ("left", "right")}:
            bcs = [["periodic", "periodic"], ["periodic", "periodic"]]  # doubly periodic (euler_wave.py)
        elif nd == 1:  # 1D (Sod_shock_tube.py, shu_osher.py): a Dirichlet face at x0 = 0
            if other or bcs[0][0] != "dirichlet" or bcs[0][1] not in ("dirichlet", "extrapolation"):
                raise NotImplementedError("1D Euler block boundary conditions: %s" %
                                          (other or sorted(n for n in names if "boundary dir" in n)))
            bcs[1] = ["periodic", "periodic"]
        elif other or bcs[1][0] != "symmetry" or None in bcs[0] or bcs[1][1] is None:
            raise NotImplementedError("2D Euler block boundary conditions: %s" %
                                      (other or sorted(n for n in names if "boundary dir" in n)))
        physics_check.check_algorithm(self.components, nd, viscous=False, metric=False)
        self._euler_faces = bcs
        plan = Plan(ndim=nd, n=(64, 32, 1) if nd == 2 else (64, 1, 1), delta=(1.0, 1.0, 1.0), conv=conv,
                    weno_eps=1e-14 if conv == "weno5z" else 1e-6,  # WenoZ.eps / WenoJS.eps (weno.py)
                    visc="none", rk=rk, precision=precision, averaging=averaging, x1_grid="uniform",
                    bc=(tuple(bcs[0]), tuple(bcs[1]), ("periodic", "periodic")),
                    rk_a=rk_a, rk_b=rk_b, use_graphs=use_graphs, ic="host",
                    name="euler%dd" % nd, kernels=[n for n in names if n])
        return self._euler_states(plan)

    def _euler_states(self, plan):
        """The Dirichlet states of a 2D Euler block's faces with the plan's constants."""
        consts = {"gama": plan.gama, "Minf": plan.Minf}
        consts.update({k: v for k, v in self.values.items() if isinstance(v, (int, float))})
        b = self._euler_faces
        nd = plan.ndim
        kw = {}
        x0 = []
        for side in range(2):
            if b[0][side] == "dirichlet":
                lo, hi, xs = self._face_states("Dirichlet boundary dir0 side%d" % side, consts, nd)
                if xs != 1e300:
                    raise NotImplementedError("Dirichlet x0 face: a constant state expected")
                x0.append(lo)
            else:
                x0.append((0.0,) * (nd + 2))
        kw["dirichlet_x0"] = tuple(x0) if "dirichlet" in b[0] else None
        if b[1][1] == "dirichlet":
            lo, hi, xs = self._face_states("Dirichlet boundary dir1 side1", consts)
            kw.update(dirichlet_lo=lo, dirichlet_hi=hi, dirichlet_x_switch=xs)
        return plan.replace(**kw)

    def _power_law_viscosity(self):
        """The viscosity relation of the CRmu kernel: None for Sutherland's law (katzer_SBLI.py:25,
        checked with the other relations), else the exponent a of mu = T^a
        (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:30)."""
        import sympy
        eqs = [e for k in self._kernels("CRmu") for e in k.equations if str(getattr(e.lhs, "base", "")) == "mu_B0"]
        if len(eqs) != 1:
            raise NotImplementedError("viscosity: one relation for mu expected")
        r = eqs[0].rhs
        if isinstance(r, sympy.Pow) and type(r.base).__name__ == "DataSet" and str(r.base.base) == "T_B0" and \
                all(int(i) == 0 for i in r.base.indices) and r.exp.is_number:
            return float(r.exp)
        return None

    def _forcing(self, reconstruction):
        """The constant forcing of turbulent_channel.py:15-16 (- KD(_i,_j) c_j in the momentum
        equations, - Dot(c_j, u_j) in the energy equation): the constants c0, c1, c2 of the
        characteristic residual kernel (their form is checked by physics_check).  Returns None without
        them, else their values as far as the algorithm knows them (the simulation parameters complete
        them)."""
        import sympy
        found = {}
        for k in self._kernels(""):
            if not re.match(r"LLF(Weno|Teno) Residual", (k.computation_name or "").strip()):
                continue
            for e in k.equations:
                for a in sympy.preorder_traversal(e.rhs):
                    if type(a).__name__ == "ConstantObject" and re.fullmatch(r"c[0-2]", str(a)):
                        found[int(str(a)[1])] = a
        if not found:
            return None
        if len(found) != self.block.ndim:
            raise NotImplementedError("forcing: constants %s" % sorted("c%d" % d for d in found))
        vals = [getattr(found[d], "value", None) for d in range(3)]
        return tuple(float(v) if isinstance(v, (int, float)) else 0.0 for v in vals)

    def _body_force(self):
        """Recognise the body force of apps/transitional_SBLI/transitional_SBLI.py:80-89: a constituent
        relation BF = A exp(-((x0-xF)^2 + (x1-yF)^2)) cos(bta x2) sin(omega dt iter) of the coordinate
        arrays and the iteration number, added to the continuity equation's residual.  Returns None
        without one, else (A, xF, yF, bta, omega) (values as far as the algorithm knows them; the
        simulation parameters complete them)."""
        import math
        import random
        import sympy
        eqs = [(k, e) for k in self.components if type(k).__name__ == "Kernel" for e in k.equations
               if str(getattr(e.lhs, "base", "")) == "BF_B0"]
        if not eqs:
            return None
        if len(eqs) != 1:
            raise NotImplementedError("body force: written more than once")
        e = eqs[0][1]
        syms = {}
        it = sympy.preorder_traversal(e.rhs)
        for a in it:
            t = type(a).__name__
            if t == "DataSet":
                it.skip()  # not its shape constants
                if any(int(i) != 0 for i in a.indices) or str(a.base) not in ("x0_B0", "x1_B0", "x2_B0"):
                    raise NotImplementedError("body force reads %s" % a)
                syms[a] = sympy.Symbol("_bf_" + str(a.base)[:2])
            elif t == "ConstantObject":
                if str(a) not in self._BF_CONSTS + ("dt",):
                    raise NotImplementedError("body force constant %s" % a)
                syms[a] = sympy.Symbol("_bf_" + str(a))
            elif t == "Globalvariable":
                if str(a) != "iter":
                    raise NotImplementedError("body force reads %s" % a)
                syms[a] = sympy.Symbol("_bf_iter")
        f = e.rhs.xreplace(syms)
        rnd = random.Random(11)
        for _ in range(6):
            v = {n: rnd.uniform(0.1, 2.0) for n in ("x0", "x1", "x2", "A", "xF", "yF", "bta", "omega", "dt")}
            v["iter"] = float(rnd.randint(0, 50))
            want = v["A"] * math.exp(-(v["x0"] - v["xF"]) ** 2 - (v["x1"] - v["yF"]) ** 2) * \
                math.cos(v["bta"] * v["x2"]) * math.sin(v["omega"] * v["dt"] * v["iter"])
            got = float(f.subs({sympy.Symbol("_bf_" + n): x for n, x in v.items()}))
            if abs(got - want) > 1e-12 * max(1.0, abs(want)):
                raise NotImplementedError("body force: formula not recognised")
        # the continuity residual must add BF once (the generated residual kernel's "+ BF_B0")
        adds = [k for k in self.components if type(k).__name__ == "Kernel" for q in k.equations
                if str(getattr(q.lhs, "base", "")) == "Residual0_B0" and "BF_B0" in str(q.rhs)]
        if len(adds) != 1:
            raise NotImplementedError("body force: not added to the continuity equation exactly once")
        vals = {str(a): getattr(a, "value", None) for a in syms if type(a).__name__ == "ConstantObject"}
        return tuple(float(vals[k]) if isinstance(vals.get(k), (int, float)) else 0.0 for k in self._BF_CONSTS)

    def _closures_2d(self, periodic0=False):
        """The one-sided closure each face applies to the central derivatives of its direction
        (opensblifunctions.py:523-534 wraps every central derivative in a Piecewise over the grid
        index): ReducedAccess closes the first two points of a face (reduced_access_scheme.py:34-83),
        Carpenter, the default of every face class, the first four (Carpenter_scheme.py:61-78).  Read
        from the conditions of those Piecewise expressions in the algorithm's kernels."""
        import sympy
        from sympy import preorder_traversal
        depth = {(d, side): 0 for d in range(2) for side in range(2)}
        for k in self._kernels(""):
            for e in k.equations:
                for a in preorder_traversal(e.rhs):
                    if not isinstance(a, sympy.Piecewise):
                        continue
                    for _, cond in a.args:
                        if not isinstance(cond, sympy.Equality):
                            continue
                        # idx[d] == loc or idx[d] == block0npd - m, in either orientation
                        e = sympy.expand(cond.lhs - cond.rhs)
                        ix = [x for x in e.atoms(sympy.Indexed) if str(x.base) == "idx"]
                        if len(ix) != 1:
                            continue
                        m = re.match(r"idx\[(\d)\]$", str(ix[0]))
                        if not m or int(m.group(1)) > 1:
                            continue
                        d, k = int(m.group(1)), e.coeff(ix[0])
                        if k not in (1, -1):
                            continue
                        r = sympy.expand(-(e - k * ix[0]) / k)
                        if r.is_Integer:
                            depth[(d, 0)] = max(depth[(d, 0)], int(r) + 1)
                        elif {str(x) for x in r.free_symbols} == {"block0np%d" % d}:
                            npd = next(iter(r.free_symbols))
                            depth[(d, 1)] = max(depth[(d, 1)], int(npd - r))
        kinds = {0: "none", 2: "reduced_access", 4: "carpenter"}  # none: a symmetry face's mirrored halos
        out = []
        for d in range(2):
            if d == 0 and periodic0:  # no closure on a periodic axis (the field is unused there)
                if depth[(0, 0)] or depth[(0, 1)]:
                    raise NotImplementedError("periodic x0 with one-sided derivative closures")
                out.append(("carpenter", "carpenter"))
                continue
            pair = []
            for side in range(2):
                if depth[(d, side)] not in kinds:
                    raise NotImplementedError("face dir%d side%d: one-sided closure of %d points is not lowered"
                                              % (d, side, depth[(d, side)]))
                pair.append(kinds[depth[(d, side)]])
            out.append(tuple(pair))
        return tuple(out)

    def _adaptive_teno(self, teno):
        """Recognise the adaptive TENO cut-off (LLFTeno(formulation='adaptive'), schemes/spatial/
        teno.py:430-443) and the modified Ducros sensor it reads (schemes/spatial/shock_sensors.py:
        12-49, added to the constituent relations).  Returns None for a fixed C_T, else the sensor's
        epsilon (the value the generator gives the constant; a value substituted for it as a
        simulation parameter does not reach the generated code, whose line is not `epsilon=Input;`).
        Both formulas are checked numerically against the forms the GPU kernel implements."""
        import math
        import random
        import sympy
        ct = [e for k in teno for e in k.equations if str(e.lhs) == "TENO_CT"]
        if not ct:
            if any("TENO" in str(e.rhs) and "TENO_CT" not in str(e.rhs) for k in teno for e in k.equations):
                raise NotImplementedError("TENO cut-off form not recognised")
            return None
        sensor = None
        for e in ct:
            ds = [a for a in sympy.preorder_traversal(e.rhs) if type(a).__name__ == "DataSet"]
            names = {str(a.base) for a in ds}
            if len(names) != 1 or any(int(i) != 0 for a in ds for i in a.indices):
                raise NotImplementedError("adaptive TENO: C_T must read one sensor array at the interface's left point")
            name = names.pop()
            if sensor not in (None, name):
                raise NotImplementedError("adaptive TENO: one sensor array for both directions expected")
            sensor = name
            th, a1, a2 = sympy.symbols("_osb_th _osb_a1 _osb_a2")
            reps = {a: th for a in ds}
            for a in sympy.preorder_traversal(e.rhs):
                if str(a) == "teno_a1":
                    reps[a] = a1
                elif str(a) == "teno_a2":
                    reps[a] = a2
            f = e.rhs.xreplace(reps)
            if f.free_symbols - {th, a1, a2}:
                raise NotImplementedError("adaptive TENO: unexpected symbols in C_T: %s" % (f.free_symbols - {th, a1, a2}))
            for t in (0.0, 0.013, 0.31, 0.5, 0.77, 0.999, 1.0):
                want = 10.0 ** (-math.floor(10.5 - 4.5 * (1 - (1 - t) ** 4 * (4 * t + 1))))
                got = float(f.subs({th: t, a1: 10.5, a2: 4.5}))
                if abs(got - want) > 1e-12 * want:
                    raise NotImplementedError("adaptive TENO: C_T formula not recognised")
        # the sensor equation, with its velocity derivatives classified by the variable and direction
        # of their interior (default-branch) central stencil: locals (GridVariables) of the sensor's
        # kernel on 2D blocks, work arrays written by the "ConstituentRelations CD" kernels on 3D blocks
        locs, theta_eq = {}, None
        for k in self.components:
            if type(k).__name__ != "Kernel":
                continue
            for e in k.equations:
                if str(e.lhs) == sensor or str(getattr(e.lhs, "base", "")) == sensor:
                    if theta_eq is not None:
                        raise NotImplementedError("adaptive TENO: sensor written more than once")
                    theta_eq, kern = e, k
        if theta_eq is None:
            raise NotImplementedError("adaptive TENO: no kernel evaluates the sensor %s" % sensor)

        def classify(rhs, what):
            body = rhs.args[-1][0] if isinstance(rhs, sympy.Piecewise) else rhs
            ds = [a for a in sympy.preorder_traversal(body) if type(a).__name__ == "DataSet"]
            var = {str(a.base) for a in ds}
            dirs = {d for a in ds for d, i in enumerate(a.indices) if int(i) != 0}
            offs = sorted({int(i) for a in ds for i in a.indices if int(i) != 0})
            if len(var) != 1 or len(dirs) != 1 or offs != [-2, -1, 1, 2]:
                raise NotImplementedError("adaptive TENO: sensor derivative %s not recognised" % what)
            return var.pop(), dirs.pop()

        for e in kern.equations:
            # derivative locals: a closure Piecewise, or (periodic axes) a plain central stencil
            if type(e.lhs).__name__ == "GridVariable" and (
                    isinstance(e.rhs, sympy.Piecewise) or
                    any(type(a).__name__ == "DataSet" and any(int(i) != 0 for i in a.indices)
                        for a in sympy.preorder_traversal(e.rhs))):
                locs[e.lhs] = classify(e.rhs, e.lhs)
        nd = self.block.ndim
        # work arrays: the last write before the sensor kernel, by a sensor-derivative kernel
        written = {}
        for k in self.components:
            if k is kern:
                break
            if type(k).__name__ != "Kernel":
                continue
            for e in k.equations:
                if hasattr(e.lhs, "base"):
                    written[str(e.lhs.base)] = (k, e)
        sym = {}
        for v in range(nd):
            for d in range(nd):
                sym[("u%d_B0" % v, d)] = sympy.Symbol("_osb_d_u%d_%d" % (v, d))
        D = sympy.Symbol("_osb_D11")
        reps, eps = {}, None
        for a in sympy.preorder_traversal(theta_eq.rhs):
            t = type(a).__name__
            if t == "GridVariable":
                if a not in locs:
                    raise NotImplementedError("adaptive TENO: sensor local %s not recognised" % a)
                reps[a] = sym[locs[a]]
            elif t == "DataSet" and str(a.base) == "D11_B0" and all(int(i) == 0 for i in a.indices):
                reps[a] = D
            elif t == "DataSet":
                w = written.get(str(a.base))
                if (nd != 3 or w is None or any(int(i) != 0 for i in a.indices)
                        or not (w[0].computation_name or "").startswith("ConstituentRelations CD")):
                    raise NotImplementedError("adaptive TENO: sensor input %s not recognised" % a)
                key = classify(w[1].rhs, a)
                if key not in sym:
                    raise NotImplementedError("adaptive TENO: sensor input %s is not a velocity derivative" % a)
                reps[a] = sym[key]
            elif t == "ConstantObject" and str(a) == "epsilon":
                eps = float(a.value)
                reps[a] = sympy.Float(eps)
        g = theta_eq.rhs.xreplace(reps)
        # the derivative locals carry inv_0/inv_1 = 1/Delta; take Delta = 1 for the check (the work
        # arrays' stencils and spacing factors are checked with the other derivative kernels)
        g = g.subs({s_: 1 for s_ in g.free_symbols if str(s_) in ("inv_0", "inv_1")})
        if eps is None or g.free_symbols - set(sym.values()) - {D}:
            raise NotImplementedError("adaptive TENO: sensor formula not recognised")
        # compare against the sensor the GPU kernel implements on random derivative values: D11 is
        # the metric factor d(xi1)/d(x1) of a block stretched in x1, 1 on a Cartesian block
        rnd = random.Random(7)
        metric = D in g.free_symbols
        for _ in range(8):
            vals = {k_: rnd.uniform(-0.02, 0.02) for k_ in sym}
            Dv = rnd.uniform(0.5, 2.0) if metric else 1.0
            du = [[vals[("u%d_B0" % c, d)] * (Dv if d == 1 else 1.0) for d in range(nd)] for c in range(nd)]
            div = sum(du[c][c] for c in range(nd))
            if nd == 2:
                om2 = (du[1][0] - du[0][1]) ** 2
            else:
                om2 = (du[2][1] - du[1][2]) ** 2 + (du[0][2] - du[2][0]) ** 2 + (du[1][0] - du[0][1]) ** 2
            want = (0.5 - 0.5 * math.tanh(2.5 + 250.0 * div)) * div * div / (eps + div * div + om2)
            got = float(g.subs({**{sym[k_]: vals[k_] for k_ in sym}, D: Dv}))
            if abs(got - want) > 1e-12 * max(abs(want), 1e-300):
                raise NotImplementedError("adaptive TENO: sensor formula not recognised")
        return eps

    # ------------------------------------------------------------------ constants
    def substitute_simulation_parameters(self, constants, values):
        """Same arguments as opensbli.utilities.helperfunctions.substitute_simulation_parameters."""
        env = {}
        for c, v in zip(constants, values):
            env[c] = _eval_c_expr(str(v), env) if isinstance(v, str) else v
        self.values.update(env)
        p = self.plan
        nd = p.ndim
        n = tuple(int(env.get("block0np%d" % d, p.n[d])) if d < nd else 1 for d in range(3))
        delta = tuple(float(env.get("Delta%dblock0" % d, p.delta[d])) if d < nd else 1.0 for d in range(3))
        kw = dict(n=n, delta=delta, gama=float(env.get("gama", p.gama)), Minf=float(env.get("Minf", p.Minf)),
                  Re=float(env.get("Re", p.Re)), Pr=float(env.get("Pr", p.Pr)),
                  dt=float(env["dt"]) if "dt" in env else p.dt,
                  niter=int(env["niter"]) if "niter" in env else p.niter)
        if nd == 3 and p.conv in ("teno5", "teno6"):
            kw.update(teno_eps=float(env.get("eps", p.teno_eps)), teno_ct=float(env.get("TENO_CT", p.teno_ct)))
        if p.body_force is not None:
            kw["body_force"] = tuple(float(env.get(k, v)) for k, v in zip(self._BF_CONSTS, p.body_force))
        if p.forcing is not None:
            kw["forcing"] = tuple(float(env.get("c%d" % d, v)) for d, v in enumerate(p.forcing))
        if p.x1_grid == "tanh":
            kw["stretch"] = float(env.get("stretch", p.stretch))
        if p.rk == "ls_rk3":  # wall-bounded blocks
            kw.update(Twall=float(env.get("Twall", p.Twall)), SuthT=float(env.get("SuthT", p.SuthT)),
                      RefT=float(env.get("RefT", p.RefT)), teno_eps=float(env.get("eps", p.teno_eps)),
                      teno_ct=float(env.get("TENO_CT", p.teno_ct)), Lx1=float(env.get("Lx1", p.Lx1)),
                      by=float(env.get("by", p.by)), teno_a1=float(env.get("teno_a1", p.teno_a1)),
                      teno_a2=float(env.get("teno_a2", p.teno_a2)))
        self.plan = p.replace(**kw)
        if p.visc == "const" and p.ndim == 2 and float(env.get("mu", 1.0)) != 1.0:
            raise NotImplementedError("Cartesian viscous blocks: the kernels implement mu = 1, the script sets %s"
                                      % env.get("mu"))
        if p.visc == "none" and p.ndim <= 2:  # the Dirichlet states of an Euler block use gama and Minf
            self.plan = self._euler_states(self.plan)
        return self.plan

    # ------------------------------------------------------------------ initial condition
    def initial_fields(self, halo=0):
        """Evaluate the script's GridBasedInitialisation kernel (initialisation/gridbasedinit.py:15-57)
        with numpy, in the kernel's equation order, on the interior plus `halo` points on every side.
        Returns {name: FP64 array [z][y][x] (2D: [y][x])} for every array the kernel assigns."""
        import numpy as np
        import sympy
        k = self.ic_kernel
        if k is None:
            raise NotImplementedError("no Grid_based_initialisation kernel in the algorithm")
        p = self.plan
        nd = p.ndim
        ranges = [np.arange(-halo, p.n[d] + halo, dtype=np.float64) for d in range(nd)]
        grids = np.meshgrid(*ranges[::-1], indexing="ij")  # [z][y][x] order
        grid_idx = grids[::-1]                               # grid_idx[d] varies along axis d
        shape = grids[0].shape
        env = {}
        consts = dict(self.values)
        consts.update({"gama": p.gama, "Minf": p.Minf, "Re": p.Re, "Pr": p.Pr})
        for d in range(3):
            consts["Delta%dblock0" % d] = p.delta[d]
        if p.rk == "ls_rk3":  # wall-bounded blocks (2D, or 3D with a periodic x2)
            consts.update({"Lx1": p.Lx1, "by": p.by, "Twall": p.Twall, "SuthT": p.SuthT, "RefT": p.RefT})
        out = {}
        for eq in k.equations:
            rhs = eq.rhs
            reps = {}
            for a in sympy.preorder_traversal(rhs):
                t = type(a).__name__
                if t == "Grididx":
                    reps[a] = sympy.Symbol("_osb_gi%d" % int(a.number))
                elif t == "DataSet":
                    reps[a] = sympy.Symbol("_osb_ds_" + re.sub(r"_B0$", "", str(a.base)))
            rhs = rhs.xreplace(reps)
            subs_syms, args = [], []
            for sym in rhs.free_symbols:
                name = str(sym)
                if name.startswith("_osb_gi"):
                    subs_syms.append(sym); args.append(grid_idx[int(name[7:])])
                elif name.startswith("_osb_ds_"):
                    subs_syms.append(sym); args.append(env[name[8:]])
                elif name in env:
                    subs_syms.append(sym); args.append(env[name])
                elif name in consts:
                    subs_syms.append(sym); args.append(consts[name])
                else:
                    raise NotImplementedError("initial condition symbol %s has no value" % name)
            f = sympy.lambdify(subs_syms, rhs, "numpy")
            val = np.broadcast_to(np.asarray(f(*args), dtype=np.float64), shape).copy()
            lhs = eq.lhs
            name = re.sub(r"_B0$", "", str(lhs.base) if hasattr(lhs, "base") else str(lhs))
            env[name] = val
            out[name] = val
        return out

    def state_names(self):
        return {1: ["rho", "rhou0", "rhoE"], 2: ["rho", "rhou0", "rhou1", "rhoE"]}.get(
            self.plan.ndim, ["rho", "rhou0", "rhou1", "rhou2", "rhoE"])

    def initial_state(self, halo=0):
        """FP64 initial conserved state [nvar][...] from the script's initialisation kernel."""
        import numpy as np
        out = self.initial_fields(halo)
        order = self.state_names()
        missing = [v for v in order if v not in out]
        if missing:
            raise NotImplementedError("initialisation does not set %s" % missing)
        return np.stack([out[v] for v in order])

    # ------------------------------------------------------------------ execution
    def solver(self, device=None):
        from .runtime import Solver
        return Solver(self.plan, device=device)

    def io_requests(self):
        """The block's HDF5 IO objects (core/io_hdf5.py:19-132) as plain data: a list of
        {"kind": "write"|"read", "arrays": [dat names], "every": N or None, "at_end": bool,
        "name": file name or None}."""
        out, seen = [], set()
        # the IO objects sit in the algorithm's program where the generated code calls them
        for io in self.components:
            if type(io).__name__ != "iohdf5" or id(io) in seen:
                continue
            seen.add(id(io))
            kw = getattr(io, "kwargs", {}) or {}
            places = getattr(io, "algorithm_place", []) or []
            every = [getattr(p, "frequency", None) for p in places if type(p).__name__ == "InTheSimulation"]
            r = {"kind": kw.get("iotype", "write"), "arrays": [str(a) for a in io.arrays],
                 "every": int(every[0]) if every and every[0] else None,
                 "at_end": any(type(p).__name__ == "AfterSimulationEnds" for p in places),
                 "name": kw.get("name") if kw.get("iotype", "write") == "write" else kw.get("filename", "data.h5")}
            if r not in out:  # the program lists an IO object once per place it acts at
                out.append(r)
        return out

    def _output_dats(self, s, names, coords):
        """The dats of `names` this library can produce, as FP64 interior arrays: conserved variables
        (written by Solver.write_ops_hdf5 itself), x0/x1 of the grid, and on 2D blocks with adaptive TENO
        the cut-off field TENO_B0.  Returns (extra dats, names it cannot produce)."""
        extra, skipped = {}, []
        conserved = set(s.state_names())
        for n in names:
            if n in conserved:
                continue
            base = n[:-3] if n.endswith("_B0") else n
            if base in coords:
                extra[n] = coords[base]
            elif n == "TENO_B0" and self.plan.teno_adaptive:
                extra[n] = s.teno_cutoff().cpu().numpy()
            else:
                skipped.append(n)
        return extra, skipped

    def run(self, niter=None, dt=None, device=None, monitor=None, output_dir=None):
        """Initialise from the script's initial condition and advance niter steps (defaults: the
        script's niter and dt).  The algorithm's SimulationMonitor, if it has one (or `monitor`, an
        opensbli_gb300.monitor.SimulationMonitor), samples and prints where the generated code would.
        With `output_dir`, the script's HDF5 IO is carried out there as the generated code does it:
        read requests (iotype "read") set the state from their file before the first step; write
        requests write opensbli_output_%06d.h5 every `save_every` steps and opensbli_output.h5 (or the
        requested name) after the last, in the OPS block layout (opensbli_gb300.hdf5).  Dats the
        library does not hold are left out and listed in `self.skipped_output`.
        Returns the Solver, whose state64() gives the FP64 state."""
        import os
        from . import monitor as mon
        s = self.solver(device)
        coords = {}
        if self.plan.ndim == 1:
            f = self.initial_fields(halo=4)
            s.set_state64_padded(np.stack([f[v] for v in self.state_names()]), 4)
            coords = {k: f[k][4:-4] for k in ("x0",) if k in f}
        elif self.plan.ndim == 2:
            f = self.initial_fields(halo=4)
            if self.plan.x1_grid != "uniform":
                s.set_coordinate(f["x1"], 4)
            s.set_state64_padded(np.stack([f[v] for v in self.state_names()]), 4)
            coords = {k: f[k][4:-4, 4:-4] for k in ("x0", "x1") if k in f}
        elif self.plan.rk == "ls_rk3":  # 3D wall-bounded: x1 is a function of j alone
            f = self.initial_fields(halo=3)
            s.set_coordinate(f["x1"][3, :, 3], 3)
            s.set_state64_padded(np.stack([f[v] for v in self.state_names()]), 3)
            coords = {k: f[k][3:-3, 3:-3, 3:-3] for k in ("x0", "x1", "x2") if k in f}
        else:
            s.set_state64(self.initial_state())
        ios = self.io_requests() if output_dir is not None else []
        for r in ios:
            if r["kind"] == "read":
                s.read_ops_hdf5(os.path.join(output_dir, r["name"]))
        if monitor is None and getattr(self.algorithm, "simulation_monitor", None) is not None:
            monitor = mon.SimulationMonitor.from_reference(self.algorithm.simulation_monitor)
        n = int(niter if niter is not None else self.plan.niter)
        step = float(dt if dt is not None else self.plan.dt)
        writes = [r for r in ios if r["kind"] == "write"]
        self.skipped_output = []

        def write(r, fname):
            extra, skipped = self._output_dats(s, r["arrays"], coords)
            self.skipped_output += [x for x in skipped if x not in self.skipped_output]
            s.write_ops_hdf5(os.path.join(output_dir, fname), extra=extra)

        # chunks end where a periodic write is due (generated code: fmod(iter + 1, save_every) == 0)
        ends = sorted({k for r in writes if r["every"] for k in range(r["every"], n + 1, r["every"])} | {n})
        it = 0
        for e in ends:
            if e > it:
                mon.run(s, e - it, step, monitor, t0_iteration=it)
                it = e
            for r in writes:
                if r["every"] and e % r["every"] == 0 and e > 0:
                    write(r, "opensbli_output_%06d.h5" % e)
        for r in writes:
            if r["at_end"]:
                name = r["name"] or "opensbli_output"
                write(r, name if name.endswith(".h5") else name + ".h5")
        if monitor is not None:
            monitor.close()
        return s
