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
from opensbli_gb300.plan import katzer_plan, tgv_plan
from opensbli_gb300.runtime import Solver

pytestmark = pytest.mark.gpu

RED = {"ke": 0, "enstrophy": 1, "nancheck": 2}
OSB_EINVAL = -1
OSB_EUNSUPPORTED = -2
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
    # warm-up call: its first use on the device looks up the scratch address
    assert f(ctypes.byref(desc), ptrs, RED["ke"], ctypes.c_void_p(out.data_ptr()),
             ctypes.c_void_p(s.stream.cuda_stream)) == 0
    s.stream.synchronize()
    for call in range(2):
        for what in ("ke", "enstrophy", "nancheck"):
            expect = s.reduce(what)  # synchronises the solver stream
            torch.cuda.synchronize()
            allocs = torch.cuda.memory_stats(s.device).get("allocation.all.allocated", 0)
            free0, _ = torch.cuda.mem_get_info(s.device)
            rc = f(ctypes.byref(desc), ptrs, RED[what], ctypes.c_void_p(out.data_ptr()),
                   ctypes.c_void_p(s.stream.cuda_stream))
            assert rc == 0
            s.stream.synchronize()
            # the call allocated nothing: neither through torch's allocator nor from the driver
            assert torch.cuda.memory_stats(s.device).get("allocation.all.allocated", 0) == allocs
            assert torch.cuda.mem_get_info(s.device)[0] == free0
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


def test_reduce_noalloc_rejects_2d_plans():
    """2D blocks have four conserved arrays and no z-halo; the call must refuse them before it looks
    at any pointer (the dummy pointers here would fault if a kernel read them)."""
    f = entry()
    desc = runtime.make_plan_desc(katzer_plan(64, 32))
    ptrs = (ctypes.c_void_p * 5)(*([1 << 20] * 5))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for what in RED.values():
        assert f(ctypes.byref(desc), ptrs, what, ctypes.c_void_p(out.data_ptr()), None) == OSB_EUNSUPPORTED


def test_reduce_noalloc_rejects_host_output():
    """dev_out must be device memory of the current device; a host address is refused, not written."""
    f = entry()
    plan = tgv_plan(16)
    s = Solver(plan)
    s.init_tgv()
    desc = runtime.make_plan_desc(plan)
    ptrs = (ctypes.c_void_p * 5)(*[t.data_ptr() for t in s.fields])
    host = (ctypes.c_double * 1)(-1.0)
    rc = f(ctypes.byref(desc), ptrs, RED["ke"], ctypes.cast(host, ctypes.c_void_p), None)
    assert rc == OSB_EINVAL and host[0] == -1.0
    s.close()
