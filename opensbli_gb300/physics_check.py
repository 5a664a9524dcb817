"""Numerical check that the physics of a lowered algorithm is the physics the fused kernels implement.

GB300Writer recognises kernel families by name and stencil shape; a problem script with other
constituent relations, another stress or heat-flux model or another convective form could keep the
same kernel names.  This module evaluates the reference's own kernel equations (the SymPy right-hand
sides in alg.prg, core/kernel.py:62-230) at random values and compares them with the formulas of the
fused kernels:

* constituent relations (taylor_green_vortex.py:30-32, katzer_SBLI.py:21-25): u_i = rhou_i / rho,
  p = (gama-1)(rhoE - |rhou|^2 / (2 rho)), T = gama Minf^2 p / rho, a = sqrt(gama p / rho) and the
  Sutherland viscosity mu = T^1.5 (1 + S) / (T + S), S = SuthT / RefT;
* central derivative kernels (opensblifunctions.py:485-521): 4th-order first and second derivative
  weights (interior branch) and their 1/delta factors, nested first derivatives for mixed ones;
* the convective skew-symmetric residual (parsing.py:75-111) and the viscous residual with the
  Newtonian stress tau_ij = (mu/Re)(d_j u_i + d_i u_j - 2/3 delta_ij d_k u_k) and the Fourier heat
  flux k dT/dx_j, k = mu / ((gama-1) Minf^2 Pr Re), with the metric transform of an x1-stretched
  block (metric.py:37-234): d/dx1 = D11 d/dxi1, d2/dx1^2 = D11^2 d2/dxi1^2 + D11 SD111 d/dxi1;
* the characteristic-flux residual: R = -sum_d (F_d[i] - F_d[i-1]) / delta_d (times D11 along x1).

Derivative work arrays are reused within a stage (the generator hands out wk0, wk1, ... per kernel),
so the meaning of each array is followed in program order.  Any mismatch raises NotImplementedError.
"""
import math
import random
import re

import sympy

_DERIV_NAMES = re.compile(r"^(Convective|Viscous|Derivative evaluation|ConstituentRelations) (CD )+")


def _base(x):
    """Array name without the block suffix."""
    return re.sub(r"_B\d+$", "", str(x.base if hasattr(x, "base") else x))


def _leaves(expr):
    """DataSet, ConstantObject and GridVariable atoms of expr (a DataSet's own arguments, its shape
    constants, are not visited)."""
    out = []
    it = sympy.preorder_traversal(expr)
    for a in it:
        if type(a).__name__ in ("DataSet", "ConstantObject", "GridVariable"):
            out.append(a)
            it.skip()
    return out


def _datasets(expr):
    return [a for a in _leaves(expr) if type(a).__name__ == "DataSet"]


def _constants(expr):
    return [a for a in _leaves(expr) if type(a).__name__ == "ConstantObject"]


def _interior(expr):
    """expr with every Piecewise over grid indices (the one-sided boundary closures) replaced by its
    default (last) branch: the interior stencil."""
    return expr.replace(lambda x: isinstance(x, sympy.Piecewise), lambda x: x.args[-1][0])


class PhysicsCheck:
    """Evaluate the kernels of `components` (alg.prg walked in program order) against the built-in
    formulas of a 3D block with constant viscosity, or a 2D or 3D block stretched in x1 with Sutherland
    viscosity."""

    def __init__(self, components, ndim, viscous, sutherland=False, metric=False, skew=False, body_force=False,
                 visc_exp=None, forcing=False):
        self.components = [c for c in components if type(c).__name__ == "Kernel"]
        self.ndim, self.viscous, self.sutherland, self.metric, self.skew = ndim, viscous, sutherland, metric, skew
        self.body_force, self.visc_exp, self.forcing = body_force, visc_exp, forcing
        self.rnd = random.Random(2024)
        self.delta = (0.37, 0.53, 0.61)  # test spacings for the 1/delta factors
        # test values; mu is a script's constant viscosity, which the kernels implement as 1
        self.consts = {"gama": 1.4, "Minf": 0.7, "Re": 950.0, "Pr": 0.72, "SuthT": 110.4, "RefT": 288.0, "mu": 1.0}

    # ------------------------------------------------------------------ helpers
    def _fail(self, what):
        raise NotImplementedError("physics outside the lowered kernels: %s" % what)

    def _const_value(self, c):
        name = str(c)
        if name in self.consts:
            return self.consts[name]
        m = re.match(r"Delta(\d)block\d+$", name)
        if m:
            return self.delta[int(m.group(1))]
        if name.startswith("inv_"):
            v = getattr(c, "value", None)
            if v is None:
                self._fail("constant %s has no value" % name)
            return self._delta_value(sympy.sympify(v))
        self._fail("constant %s in a checked kernel" % name)

    def _delta_value(self, expr):
        # Delta<d>block0 -> the test spacing of axis d
        reps = {}
        for s in expr.free_symbols:
            m = re.match(r"Delta(\d)block\d+$", str(s))
            if not m:
                self._fail("constant expression %s" % expr)
            reps[s] = self.delta[int(m.group(1))]
        return float(expr.xreplace(reps))

    # ------------------------------------------------------------------ constituent relations
    def _cr_builtin(self, st):
        g, M = self.consts["gama"], self.consts["Minf"]
        rho, E = st["rho"], st["rhoE"]
        m = [st["rhou%d" % c] for c in range(self.ndim)]
        out = {"u%d" % c: m[c] / rho for c in range(self.ndim)}
        p = (g - 1) * (E - 0.5 * sum(x * x for x in m) / rho)
        out["p"] = p
        out["T"] = g * M * M * p / rho
        out["a"] = math.sqrt(g * p / rho)
        S = self.consts["SuthT"] / self.consts["RefT"]
        if self.visc_exp is not None:  # the power law (turbulent_channel.py:30)
            out["mu"] = out["T"] ** self.visc_exp
        else:
            out["mu"] = out["T"] ** 1.5 * (1 + S) / (out["T"] + S)
        return out

    def _random_state(self):
        r = self.rnd
        st = {"rho": r.uniform(0.5, 2.0)}
        for c in range(self.ndim):
            st["rhou%d" % c] = r.uniform(-1.0, 1.0)
        p = r.uniform(0.5, 2.0)
        st["rhoE"] = p / (self.consts["gama"] - 1) + 0.5 * sum(st["rhou%d" % c] ** 2
                                                                for c in range(self.ndim)) / st["rho"]
        return st

    def check_constituent_relations(self):
        seen = set()
        for k in self.components:
            cn = k.computation_name or ""
            # (the adaptive-TENO sensor kernel, "ConstituentRelations evaluation", holds stencils and is
            # checked where it is lowered)
            if not (cn.startswith("CR") or cn == "User kernel: Constituent Relations evaluation"):
                continue
            for trial in range(4):
                st = self._random_state()
                want = self._cr_builtin(st)
                env = dict(st)
                env.update(want)
                locs = {}
                for e in k.equations:
                    if type(e.lhs).__name__ == "GridVariable":
                        locs[e.lhs] = self._eval_point(e.rhs, env, locs)
                        continue
                    name = _base(e.lhs)
                    if name not in want:
                        continue
                    got = self._eval_point(e.rhs, env, locs)
                    if abs(got - want[name]) > 1e-12 * max(1.0, abs(want[name])):
                        self._fail("constituent relation for %s in %s (%.15g, expected %.15g)" % (name, cn, got,
                                                                                                want[name]))
                    seen.add(name)
        need = {"u%d" % c for c in range(self.ndim)} | {"p"}
        if self.viscous:
            need.add("T")
        if self.sutherland:
            need.add("mu")
        if not need <= seen:
            self._fail("constituent relations %s not found" % sorted(need - seen))

    def _eval_point(self, expr, env, locs):
        reps = {}
        for a in _leaves(expr):
            t = type(a).__name__
            if t == "DataSet":
                if any(int(i) != 0 for i in a.indices):
                    self._fail("stencil access in a point-wise relation: %s" % a)
                name = _base(a)
                if name not in env:
                    self._fail("point-wise relation reads %s" % name)
                reps[a] = sympy.Float(env[name], 30)
            elif t == "ConstantObject":
                reps[a] = sympy.Float(self._const_value(a), 30)
            else:
                if a not in locs:
                    self._fail("local %s used before it is set" % a)
                reps[a] = sympy.Float(locs[a], 30)
        return float(expr.xreplace(reps))

    # ------------------------------------------------------------------ derivatives and residuals
    def check_residuals(self):
        """Follow the derivative work arrays in program order and check every residual kernel."""
        meaning, products = {}, {}
        checked = set()
        for k in self.components:
            cn = (k.computation_name or "").strip()
            if cn == "Convective terms":
                # the convective terms with their derivatives evaluated locally (laminar_channel.py)
                self._check_central_residual("Convective residual", k, meaning, products)
                checked.add("Convective residual")
            elif cn.startswith("Convective terms group"):
                for e in k.equations:
                    factors = []
                    for f in sympy.Mul.make_args(e.rhs):
                        if type(f).__name__ != "DataSet" or any(int(i) != 0 for i in f.indices):
                            self._fail("product array %s" % e)
                        factors.append(_base(f))
                    products[_base(e.lhs)] = tuple(sorted(factors))
            elif _DERIV_NAMES.match(cn):
                if len(k.equations) != 1:
                    self._fail("derivative kernel %s with %d equations" % (cn, len(k.equations)))
                e = k.equations[0]
                meaning[_base(e.lhs)] = self._classify_derivative(cn, e.rhs, meaning, products)
            elif cn in ("Convective residual", "Viscous residual"):
                self._check_central_residual(cn, k, meaning, products)
                checked.add(cn)
            elif cn == "Viscous terms":
                # viscous terms with their second derivatives evaluated locally in the kernel
                self._check_central_residual("Viscous residual", k, meaning, products)
                checked.add("Viscous residual")
            elif re.match(r"LLF(Weno|Teno) Residual", cn):
                self._check_flux_residual(k)
                checked.add("flux")
        if self.skew and "Convective residual" not in checked:
            self._fail("no skew-symmetric convective residual kernel")
        if self.viscous and "Viscous residual" not in checked:
            self._fail("no viscous residual kernel")
        if not self.skew and "flux" not in checked:
            self._fail("no characteristic-flux residual kernel")

    def _classify_derivative(self, cn, rhs, meaning, products):
        body = _interior(rhs)
        ds = _datasets(body)
        bases = {_base(a) for a in ds}
        if len(bases) == 2:  # a stencil applied to the product of two arrays (laminar_channel.py's d(p u_j))
            return self._classify_product_derivative(cn, body, ds, sorted(bases))
        if len(bases) != 1:
            self._fail("derivative %s reads %s" % (cn, sorted(bases)))
        axes = {d for a in ds for d, i in enumerate(a.indices) if int(i) != 0}
        if len(axes) != 1:
            self._fail("derivative %s is not along one axis" % cn)
        d = axes.pop()
        invs = [c for c in _constants(body) if str(c).startswith("inv_")]
        if len(invs) != 1:
            self._fail("derivative %s: one 1/delta factor expected" % cn)
        inv = invs[0]
        # moments sum_o w_o o^k of the stencil weights, the inverse spacing set to 1
        mom = []
        for kpow in range(5):
            reps = {a: sympy.Integer(int(a.indices[d])) ** kpow for a in ds}
            reps[inv] = sympy.Integer(1)
            mom.append(sympy.nsimplify(body.xreplace(reps)))
        if mom == [0, 1, 0, 0, 0]:
            order = 1
        elif mom == [0, 0, 2, 0, 0]:
            order = 2
        else:
            self._fail("derivative %s: weights are not 4th-order central (moments %s)" % (cn, mom))
        want = sympy.Symbol("Delta%dblock0" % d) ** (-order)
        val = sympy.sympify(getattr(inv, "value", None))
        syms = {s: sympy.Symbol(str(s)) for s in val.free_symbols}
        if sympy.simplify(val.xreplace(syms) - want) != 0:
            self._fail("derivative %s: factor %s is not 1/Delta%d^%d" % (cn, val, d, order))
        base = bases.pop()
        if base in products:
            return (products[base], (d,) * order)
        if base in meaning:  # nested first derivative: a mixed second derivative
            inner = meaning[base]
            if order != 1 or len(inner[1]) != 1:
                self._fail("derivative %s nests more than two first derivatives" % cn)
            return (inner[0], tuple(sorted(inner[1] + (d,))))
        return ((base,), (d,) * order)

    def _classify_product_derivative(self, cn, body, ds, bases):
        """sum_o w_o f(o) g(o) along one axis, checked bilinear at random values, with the 4th-order
        central first-derivative weights: the derivative of the product f g."""
        axes = {d for a in ds for d, i in enumerate(a.indices) if int(i) != 0}
        if len(axes) != 1:
            self._fail("derivative %s is not along one axis" % cn)
        d = axes.pop()
        invs = [c for c in _constants(body) if str(c).startswith("inv_")]
        if len(invs) != 1:
            self._fail("derivative %s: one 1/delta factor expected" % cn)
        offs = sorted({int(a.indices[d]) for a in ds})
        w = {}
        for o in offs:  # f = delta(o), g = 1
            reps = {a: sympy.Integer(1 if (_base(a) == bases[1] or int(a.indices[d]) == o) and
                                     (_base(a) == bases[1] or _base(a) == bases[0]) and
                                     (_base(a) != bases[0] or int(a.indices[d]) == o) else 0) for a in ds}
            reps[invs[0]] = sympy.Integer(1)
            w[o] = sympy.nsimplify(body.xreplace(reps))
        for trial in range(3):
            vals = {(b, o): self.rnd.uniform(0.5, 1.5) for b in bases for o in offs}
            reps = {a: sympy.Float(vals[(_base(a), int(a.indices[d]))], 30) for a in ds}
            reps[invs[0]] = sympy.Integer(1)
            got = float(body.xreplace(reps))
            want = sum(float(w[o]) * vals[(bases[0], o)] * vals[(bases[1], o)] for o in offs)
            if abs(got - want) > 1e-12 * max(1.0, abs(want)):
                self._fail("derivative %s is not a stencil of the product %s" % (cn, bases))
        mom = [sympy.nsimplify(sum(w[o] * sympy.Integer(o) ** k for o in offs)) for k in range(5)]
        if mom != [0, 1, 0, 0, 0]:
            self._fail("derivative %s: weights are not 4th-order central (moments %s)" % (cn, mom))
        return (tuple(bases), (d,))

    def _point_symbols(self):
        names = ["rho", "rhoE", "p", "T", "mu", "D11", "SD111"] + ["rhou%d" % c for c in range(self.ndim)] + \
                ["u%d" % c for c in range(self.ndim)]
        return {n: sympy.Symbol("_pt_" + n) for n in names}

    def _check_central_residual(self, cn, k, meaning, products):
        pts = self._point_symbols()
        dsym = {}

        def key_symbol(key):
            if key not in dsym:
                dsym[key] = sympy.Symbol("_d_%d" % len(dsym))
            return dsym[key]

        got, local = {}, {}
        for e in k.equations:
            if type(e.lhs).__name__ == "GridVariable":  # a derivative evaluated in the kernel
                local[e.lhs] = key_symbol(self._classify_derivative("%s: %s" % (cn, e.lhs), e.rhs, meaning, products))
                continue
            lhs = _base(e.lhs)
            m = re.match(r"Residual(\d)$", lhs)
            if not m:
                self._fail("%s writes %s" % (cn, lhs))
            reps = {}
            for a in _leaves(e.rhs):
                t = type(a).__name__
                if t == "DataSet":
                    if any(int(i) != 0 for i in a.indices):
                        self._fail("%s reads %s with a stencil" % (cn, a))
                    b = _base(a)
                    if b == lhs:
                        reps[a] = sympy.Integer(0)  # the residual it adds to
                    elif b in meaning:
                        reps[a] = key_symbol(meaning[b])
                    elif b in pts:
                        reps[a] = pts[b]
                    else:
                        self._fail("%s reads %s" % (cn, b))
                elif t == "ConstantObject":
                    if self.forcing and re.fullmatch(r"c[0-2]", str(a)):
                        reps[a] = sympy.Symbol("_c%s" % str(a)[1])
                    else:
                        reps[a] = sympy.Float(self._const_value(a), 30)
                else:
                    if a not in local:
                        self._fail("%s reads the local %s" % (cn, a))
                    reps[a] = local[a]
            got[int(m.group(1))] = e.rhs.xreplace(reps)
        want = self._builtin_residual(cn, pts, key_symbol)
        if set(got) != set(want):
            self._fail("%s sets residuals %s, the kernels %s" % (cn, sorted(got), sorted(want)))
        syms = list(pts.values()) + list(dsym.values()) + \
            ([sympy.Symbol("_c%d" % k) for k in range(self.ndim)] if self.forcing else [])
        for trial in range(3):
            vals = {s: sympy.Float(self.rnd.uniform(0.3, 1.7) * self.rnd.choice((-1, 1)), 30) for s in syms}
            for v in ("rho", "p", "T", "mu", "D11"):
                vals[pts[v]] = abs(vals[pts[v]])
            for r in want:
                a, b = float(got[r].xreplace(vals)), float(want[r].xreplace(vals))
                if abs(a - b) > 1e-10 * max(1.0, abs(b)):
                    self._fail("%s: residual %d differs from the lowered formula (%.12g vs %.12g)" % (cn, r, a, b))

    def _builtin_residual(self, cn, pts, key):
        nd = self.ndim
        g, M, Re, Pr = (self.consts[c] for c in ("gama", "Minf", "Re", "Pr"))
        u = [pts["u%d" % c] for c in range(nd)]
        D11, SD = pts["D11"], pts["SD111"]

        # physical derivatives in terms of the computational ones
        def d1(f, j):
            c = key((f, (j,)))
            return D11 * c if (self.metric and j == 1) else c

        def d2(name, i, j):
            f = (name,)
            i, j = min(i, j), max(i, j)
            c = key((f, (i, j)))
            if not self.metric:
                return c
            if i == 1 and j == 1:
                return D11 ** 2 * c + D11 * SD * key((f, (1,)))
            if 1 in (i, j):  # mixed with x1: D11 times the computational derivative
                return D11 * c
            return c

        R = {}
        if cn == "Convective residual":
            def skew(phi, j):
                return sympy.Rational(1, 2) * (d1(tuple(sorted((phi, "u%d" % j))), j) + u[j] * d1((phi,), j) +
                                               pts[phi] * d1(("u%d" % j,), j))
            R[0] = -sum(skew("rho", j) for j in range(nd))
            for i in range(nd):
                R[1 + i] = -sum(skew("rhou%d" % i, j) for j in range(nd)) - d1(("p",), i)
            R[1 + nd] = -sum(skew("rhoE", j) for j in range(nd)) - sum(d1(tuple(sorted(("p", "u%d" % j))), j)
                                                                        for j in range(nd))
            if self.forcing:  # -c_i (momentum i), -c_j u_j (energy): the channels' constant forcing
                for i in range(nd):
                    R[1 + i] = R[1 + i] - sympy.Symbol("_c%d" % i)
                R[1 + nd] = R[1 + nd] - sum(sympy.Symbol("_c%d" % j) * u[j] for j in range(nd))
            return R
        mu = pts["mu"] if self.sutherland else sympy.Integer(1)
        kT = 1.0 / ((g - 1) * M * M * Pr * Re)
        du = [[d1(("u%d" % i,), j) for j in range(nd)] for i in range(nd)]
        div = sum(du[c][c] for c in range(nd))
        tau = [[du[i][j] + du[j][i] - (sympy.Rational(2, 3) * div if i == j else 0) for j in range(nd)]
               for i in range(nd)]
        dmu = [d1(("mu",), j) for j in range(nd)] if self.sutherland else [0] * nd
        # d_j tau_ij without mu: lap u_i + 1/3 d_i div u
        dtau = [sum(d2("u%d" % i, j, j) for j in range(nd)) +
                sympy.Rational(1, 3) * sum(d2("u%d" % c, i, c) for c in range(nd)) for i in range(nd)]
        mom = [(mu * dtau[i] + sum(tau[i][j] * dmu[j] for j in range(nd))) / Re for i in range(nd)]
        for i in range(nd):
            R[1 + i] = mom[i]
        heat = kT * (mu * sum(d2("T", j, j) for j in range(nd)) + sum(dmu[j] * d1(("T",), j) for j in range(nd)))
        R[1 + nd] = sum(u[i] * mom[i] for i in range(nd)) + \
            mu / Re * sum(tau[i][j] * du[i][j] for i in range(nd) for j in range(nd)) + heat
        return R

    def _check_flux_residual(self, k):
        pts = self._point_symbols()
        used = {}
        for e in k.equations:
            lhs = _base(e.lhs)
            if not re.match(r"Residual\d$", lhs):
                self._fail("characteristic residual kernel writes %s" % lhs)
            reps, arrays = {}, {}
            for a in _leaves(e.rhs):
                t = type(a).__name__
                if t == "DataSet":
                    b = _base(a)
                    if b == "BF" and lhs == "Residual0" and self.body_force and all(int(i) == 0 for i in a.indices):
                        reps[a] = sympy.Symbol("_bf")  # the continuity equation's body force (checked by the writer)
                        continue
                    if b in pts:
                        if any(int(i) != 0 for i in a.indices):
                            self._fail("characteristic residual reads %s with a stencil" % a)
                        reps[a] = pts[b]
                        continue
                    off = tuple(int(i) for i in a.indices)
                    axes = [d for d, i in enumerate(off) if i != 0]
                    if not axes:
                        arrays.setdefault(b, set()).add(0)
                        reps[a] = sympy.Symbol("_a_%s" % b)
                    elif len(axes) == 1 and off[axes[0]] == -1:
                        arrays.setdefault(b, set()).add(axes[0] + 1)
                        reps[a] = sympy.Symbol("_b_%s" % b)
                    else:
                        self._fail("characteristic residual reads %s" % a)
                elif t == "ConstantObject":
                    if self.forcing and re.fullmatch(r"c[0-2]", str(a)):
                        reps[a] = sympy.Symbol("_c%s" % str(a)[1])  # the channel's forcing constants
                    else:
                        reps[a] = sympy.Float(self._const_value(a), 30)
                else:
                    self._fail("characteristic residual reads the local %s" % a)
            # every flux array appears at i and at i-1 along one axis, one array per axis
            dirs = {}
            for b, s in arrays.items():
                if 0 not in s or len(s) != 2:
                    self._fail("characteristic residual: flux array %s not differenced" % b)
                d = max(s) - 1
                if d in dirs:
                    self._fail("characteristic residual: two flux arrays along axis %d" % d)
                dirs[d] = b
                if b in used:
                    self._fail("characteristic residual: flux array %s used twice" % b)
                used[b] = lhs
            if sorted(dirs) != list(range(self.ndim)):
                self._fail("characteristic residual: flux differences along %s" % sorted(dirs))
            got = e.rhs.xreplace(reps)
            want = -sum((sympy.Symbol("_a_%s" % dirs[d]) - sympy.Symbol("_b_%s" % dirs[d])) / self.delta[d] *
                        (pts["D11"] if (self.metric and d == 1) else 1) for d in range(self.ndim))
            if lhs == "Residual0" and sympy.Symbol("_bf") in got.free_symbols:
                want = want + sympy.Symbol("_bf")
            if self.forcing:  # -c_i (momentum i), -c_j u_j (energy): turbulent_channel.py:15-16
                c = [sympy.Symbol("_c%d" % j) for j in range(self.ndim)]
                r = int(lhs[len("Residual"):])
                if 1 <= r <= self.ndim:
                    want = want - c[r - 1]
                elif r == self.ndim + 1:
                    want = want - sum(c[j] * pts["u%d" % j] for j in range(self.ndim))
            for trial in range(3):
                vals = {s: sympy.Float(self.rnd.uniform(-2, 2), 30) for s in got.free_symbols | want.free_symbols}
                a, b = float(got.xreplace(vals)), float(want.xreplace(vals))
                if abs(a - b) > 1e-10 * max(1.0, abs(b)):
                    self._fail("characteristic residual %s is not -sum_d dF_d/dx_d" % lhs)


def check_algorithm(components, ndim, viscous, sutherland=False, metric=False, skew=False, body_force=False,
                    visc_exp=None, forcing=False):
    """Raise NotImplementedError unless the algorithm's constituent relations, derivative stencils and
    residual kernels are the ones the fused kernels implement (see the module docstring).  body_force:
    the continuity residual may add the BF array (recognised by the writer); visc_exp: mu = T^visc_exp
    instead of Sutherland's law; forcing: the characteristic residual subtracts the constants c_i
    (momentum) and c_j u_j (energy)."""
    pc = PhysicsCheck(components, ndim, viscous, sutherland=sutherland, metric=metric, skew=skew,
                      body_force=body_force, visc_exp=visc_exp, forcing=forcing)
    pc.check_constituent_relations()
    pc.check_residuals()
