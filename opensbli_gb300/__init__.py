"""opensbli_gb300: a GB300 (sm_103a) backend for OpenSBLI's per-timestep hot path.

GB300Writer(alg) lowers a reference problem script's TraditionalAlgorithmRK to a Plan; Solver(plan)
runs it on one GPU through the C ABI of libosbli_gb300 (include/osb_gb300.h).
"""
from .plan import Plan, tgv_plan, tgv_cfl_dt  # noqa: F401
from .writer import GB300Writer  # noqa: F401

__all__ = ["Plan", "tgv_plan", "tgv_cfl_dt", "GB300Writer"]
