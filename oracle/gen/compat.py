"""SymPy-1.14 / Python-3.12 compatibility shims for running the OpenSBLI code generator.

Test infrastructure only (part of the oracle): the reference generator targets Python 2.7 and
SymPy 1.1 (README.md:29-32).  These shims supply the few names and behaviours that moved or
changed since then, so that the unmodified generator can produce its C code here.  Each shim
names the reference call site that needs it.  Nothing in the product path imports this module.
"""
import sys
import types


def _stub_module(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def install():
    """Install every shim.  Idempotent."""
    if getattr(install, "_done", False):
        return
    install._done = True

    # (1) h5py (utilities/helperfunctions.py:8) and matplotlib (utilities/katzer_init.py:6) are only
    # imported, never used on the generation path that this build exercises.
    if "h5py" not in sys.modules:
        _stub_module("h5py")
    if "matplotlib" not in sys.modules:
        mpl = _stub_module("matplotlib")
        plt = _stub_module("matplotlib.pyplot")
        plt.style = types.SimpleNamespace(use=lambda *a, **k: None)  # katzer_init.py:16 sets a style
        mpl.pyplot = plt

    import sympy
    import sympy.core

    # (2) sympy.core.compatibility.{is_sequence, exec_} (code_generation/opsc.py:7, core/parsing.py:398)
    from sympy.utilities.iterables import is_sequence

    def exec_(code, globs=None, locs=None):
        exec(code, globs, locs)

    compat = _stub_module("sympy.core.compatibility", is_sequence=is_sequence, exec_=exec_)
    sympy.core.compatibility = compat

    # (3) sympy.parsing.sympy_tokenize.{NAME, OP} (core/parsing.py:11) and
    # sympy.printing.ccode.C99CodePrinter (code_generation/opsc.py:8)
    import tokenize
    import sympy.parsing
    tok = _stub_module("sympy.parsing.sympy_tokenize", NAME=tokenize.NAME, OP=tokenize.OP)
    sympy.parsing.sympy_tokenize = tok
    from sympy.printing.c import C99CodePrinter
    import sympy.printing
    cc = _stub_module("sympy.printing.ccode", C99CodePrinter=C99CodePrinter)
    sympy.printing.ccode = cc

    # (4) calling a Symbol builds an undefined function of that name (core/parsing.py:159);
    # SymPy 1.1 had Symbol.__call__, later versions removed it.
    from sympy import Symbol, Function

    if not callable(Symbol("_probe")):
        def _symbol_call(self, *args):
            return Function(self.name)(*args)
        Symbol.__call__ = _symbol_call

    # (5) Indexed.is_commutative is assigned per instance (core/opensblifunctions.py:30); it is a
    # read-only property in current SymPy.  The override is kept in the instance dict.
    from sympy import Indexed
    from sympy.core.basic import Basic
    _base_prop = Basic.__dict__["is_commutative"]

    def _get_comm(self):
        d = self.__dict__
        if "_osb_is_commutative" in d:
            return d["_osb_is_commutative"]
        return _base_prop.__get__(self, type(self))

    def _set_comm(self, value):
        self.__dict__["_osb_is_commutative"] = value

    Indexed.is_commutative = property(_get_comm, _set_comm)

    # (6) LaTeX output is a debugging by-product (code_generation/latex.py:150-178); SymPy 1.14's
    # LaTeX printer cannot walk OpenSBLI's Grididx objects, so expressions are not written.
    from opensbli.code_generation.latex import LatexWriter

    def _write_expression(self, expression, mode=None, substitutions={}):
        return None
    LatexWriter.write_expression = _write_expression

    # (7) Grididx keeps its number as a SymPy Integer so tree traversals see a Basic
    # (core/opensbliobjects.py:503-508).
    from sympy import Integer
    from opensbli.core import opensbliobjects as _obj
    _orig_gidx_new = _obj.Grididx.__new__

    def _gidx_new(cls, label, number, **assumptions):
        if isinstance(number, int):
            number = Integer(number)
        return _orig_gidx_new(cls, label, number, **assumptions)
    _obj.Grididx.__new__ = staticmethod(_gidx_new)

    # (8) EigenSystem.generate_equations_from_matrices stores Eq objects in a Matrix
    # (schemes/spatial/shock_capturing.py:233-245), which current SymPy refuses.  Every caller
    # (:383, :467-468, :524) only iterates or flattens the result, so a row-major list with the
    # same 0 placeholders is equivalent.
    from sympy import S, factor
    from opensbli.schemes.spatial import shock_capturing as _sc
    from opensbli.equation_types.opensbliequations import OpenSBLIEq

    def _eqs_from_matrices(self, lhs_matrix, rhs_matrix):
        if lhs_matrix.shape != rhs_matrix.shape:
            raise ValueError("Matrices should have the same dimension.")
        out = []
        for no, v in enumerate(lhs_matrix):
            out.append(OpenSBLIEq(v, factor(rhs_matrix[no])) if rhs_matrix[no] != 0 else S.Zero)
        return out
    _sc.EigenSystem.generate_equations_from_matrices = _eqs_from_matrices

    # (9) MetricsEquation.generate_sd_metrics_equations zips two N-d arrays (equation_types/metric.py:
    # 207-212); SymPy 1.1 iterated them element by element, current SymPy iterates sub-arrays.
    from sympy import flatten as _flatten, Equality
    from opensbli.equation_types import metric as _metric
    from opensbli.equation_types.opensbliequations import OpenSBLIEquation

    def _sd_eqns(cls):
        def elems(a):
            return list(a.reshape(len(a)) if hasattr(a, "reshape") and hasattr(a, "shape") else _flatten(a))
        eqns = [OpenSBLIEq(x, y) for x, y in zip(elems(cls.SD_metrics), elems(cls.SD_evaluations))]
        eqns = [e for e in eqns if isinstance(e, Equality)]
        cls.sdequations = [OpenSBLIEquation(e.lhs, e.rhs) for e in eqns]
        return
    _metric.MetricsEquation.generate_sd_metrics_equations = _sd_eqns

    # (10) a GroupedPiecewise nested in an expression is printed as a Piecewise
    # (code_generation/opsc.py:48 OPSCCodePrinter; SymPy 1.1 found _print_Piecewise through the MRO).
    from opensbli.code_generation.opsc import OPSCCodePrinter
    if not hasattr(OPSCCodePrinter, "_print_GroupedPiecewise"):
        OPSCCodePrinter._print_GroupedPiecewise = OPSCCodePrinter._print_Piecewise
