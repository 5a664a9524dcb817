"""osb_reduce_noalloc: the allocation-free reduction entry point, called through the C ABI.

For callers that cannot allocate device memory where they need a diagnostic (a pool-managed host
framework, a hook between time steps): the entry point takes the state arrays and a device output
word and keeps its only scratch, per-plane partial sums, in a fixed device array.  Its results must
agree with the context-based osb_reduce within the tolerances the other GPU tests use (1e-12 for
the FP64 path, 2e-6 for the mixed path, whose osb_reduce reads the FP64 register while this entry
point reads the FP32 state), on two calls in a row with the state advanced in between.  This file
is collected last so a failure here leaves every other test already run.
"""
import ctypes

import pytest
import torch

from opensbli_gb300 import runtime
from opensbli_gb300.plan import tgv_plan
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu

RED = {"ke": 0, "enstrophy": 1, "nancheck": 2}
OSB_ETOOLARGE = -7
MAX_PLANES = 2048


def entry():
    lib = runtime.load()
    f = lib.osb_reduce_noalloc
    f.argtypes = [ctypes.POINTER(runtime.PlanDesc), ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-6)])
def test_reduce_noalloc_matches_osb_reduce(precision, tol):
    f = entry()
    plan = tgv_plan(40, conv="weno5js", Minf=1.25, precision=precision)
    s = Solver(plan)
    s.init_tgv()
    s.step(2, 2e-3)
    desc = runtime.make_plan_desc(plan)
    ptrs = (ctypes.c_void_p * 5)(*[t.data_ptr() for t in s.fields])
    out = torch.full((1,), -1.0, dtype=torch.float64, device=s.device)
    for call in range(2):
        for what in ("ke", "enstrophy", "nancheck"):
            expect = s.reduce(what)  # synchronises the solver stream
            rc = f(ctypes.byref(desc), ptrs, RED[what], ctypes.c_void_p(out.data_ptr()),
                   ctypes.c_void_p(s.stream.cuda_stream))
            assert rc == 0
            s.stream.synchronize()
            got = float(out.item())
            if what == "nancheck":
                assert got == expect == 0.0
            else:
                assert abs(got - expect) <= tol * abs(expect), (call, what, got, expect)
        s.step(1, 2e-3)  # the second call sees a different state
    s.close()


def test_reduce_noalloc_rejects_too_many_planes():
    f = entry()
    plan = tgv_plan((8, 8, MAX_PLANES + 1))
    desc = runtime.make_plan_desc(plan)
    ptrs = (ctypes.c_void_p * 5)(*([1 << 20] * 5))  # never dereferenced: the size check comes first
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert f(ctypes.byref(desc), ptrs, RED["ke"], ctypes.c_void_p(out.data_ptr()), None) == OSB_ETOOLARGE
