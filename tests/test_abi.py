"""The C ABI library: builds, loads, exports every entry point include/osb_gb300.h declares, and
validates plans on the host (no GPU needed for these)."""
import ctypes
import os
import re

import pytest

from opensbli_gb300 import runtime
from opensbli_gb300.plan import tgv_plan

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "osb_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|int64_t)\s+(osb_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    lib = runtime.load()
    syms = declared_symbols()
    assert len(syms) >= 13
    for s in syms:
        assert hasattr(lib, s), s
    assert set(runtime.EXPORTS) <= set(syms)


def layout(plan):
    lib = runtime.load()
    d = runtime.make_plan_desc(plan)
    lay = runtime.Layout()
    rc = lib.osb_query_layout(ctypes.byref(d), ctypes.byref(lay))
    return rc, lay


def test_query_layout_fp64_and_mixed():
    rc, lay = layout(tgv_plan(64))
    assert rc == 0
    assert lay.state_bytes == 8 and lay.nvar == 5
    assert tuple(lay.halo) == (4, 3, 3)
    assert lay.stride_y % 8 == 0 and lay.stride_y >= 64 + 8
    assert lay.offset == 4 + 3 * lay.stride_y + 3 * lay.stride_z
    assert lay.numel == lay.stride_z * (64 + 6)
    rc, lay = layout(tgv_plan(64, precision="mixed"))
    assert rc == 0 and lay.state_bytes == 4
    # interior rows start 16-byte aligned for FP32 state
    assert (lay.offset * 4) % 16 == 0 and (lay.stride_y * 4) % 16 == 0


def test_query_layout_accepts_adaptive_teno_on_3d():
    for conv in ("teno5", "teno6"):
        assert layout(tgv_plan(64).replace(conv=conv, teno_adaptive=True))[0] == 0


@pytest.mark.parametrize("change,code", [
    (dict(n=(4, 64, 64)), -1),                    # too small
    (dict(conv="weno5js", teno_adaptive=True), -1),  # adaptive cut-off without TENO fluxes
    (dict(visc="sutherland"), -2),
    (dict(rk="ls_rk3"), -2),
    (dict(bc=(("periodic", "symmetry"),) + (("periodic", "periodic"),) * 2), -1),
    (dict(gama=1.0), -1),
])
def test_query_layout_rejects_bad_plans(change, code):
    rc, _ = layout(tgv_plan(64).replace(**change))
    assert rc == code


def test_query_layout_2d_closures():
    from opensbli_gb300.plan import katzer_plan
    carp = (("carpenter", "carpenter"),) * 2
    assert layout(katzer_plan(64, 32, closure=carp))[0] == 0
    d = runtime.make_plan_desc(katzer_plan(64, 32))
    assert [list(r) for r in d.closure] == [[0, 0], [0, 0], [0, 0]]
    d = runtime.make_plan_desc(katzer_plan(64, 32, closure=(("reduced_access", "carpenter"),) * 2))
    assert [list(r) for r in d.closure][:2] == [[0, 1], [0, 1]]
    d.closure[1][0] = 7
    lay = runtime.Layout()
    assert runtime.load().osb_query_layout(ctypes.byref(d), ctypes.byref(lay)) == -1


def test_abi_version_mismatch():
    lib = runtime.load()
    d = runtime.make_plan_desc(tgv_plan(32))
    d.abi_version = 99
    lay = runtime.Layout()
    assert lib.osb_query_layout(ctypes.byref(d), ctypes.byref(lay)) == -1


def test_solver_refuses_without_cuda(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="CUDA"):
        runtime.Solver(tgv_plan(32))


@pytest.mark.parametrize("cname,cls", [("osb_plan_desc", runtime.PlanDesc), ("osb_layout", runtime.Layout)])
def test_ctypes_structs_match_the_header(cname, cls, tmp_path):
    """Size and every field offset of the Python descriptors equal the C compiler's for the header."""
    fields = [f[0] for f in cls._fields_]
    src = ["#include <stddef.h>", "#include <stdio.h>", '#include "osb_gb300.h"', "int main(void) {",
           '  printf("%%zu\\n", sizeof(%s));' % cname]
    src += ['  printf("%%zu\\n", offsetof(%s, %s));' % (cname, f) for f in fields]
    src += ["  return 0;", "}"]
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "probe"
    import subprocess
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(c), "-o", str(exe)])
    out = [int(x) for x in subprocess.check_output([str(exe)], text=True).split()]
    assert out[0] == ctypes.sizeof(cls)
    assert out[1:] == [getattr(cls, f).offset for f in fields]


def test_state_arrays_of_the_wrong_shape_are_refused():
    """The kernels index caller arrays from the plan's sizes, so the host refuses a mismatched array
    before any device access."""
    import torch
    runtime.Solver._check_shape(torch.zeros(5, 8, 8, 8), (5, 8, 8, 8), "state")
    with pytest.raises(ValueError, match="the block needs"):
        runtime.Solver._check_shape(torch.zeros(5, 8, 8, 7), (5, 8, 8, 8), "state")
