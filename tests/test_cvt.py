"""The integer-pipe float<->double conversions used by the mixed-precision RK update
(opensbli_gb300/csrc/osb_cvt.cuh) equal the IEEE conversions bit for bit: the header is compiled for
the host with g++ and checked against the compiler's own casts over all 2^32 floats and 2e8+
doubles (tests/native/cvt_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "opensbli_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_pipe_conversions_match_ieee(tmp_path):
    exe = str(tmp_path / "cvt_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "cvt_check.cpp"),
                           "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    bad, n = (int(v) for v in out.stdout.split())
    assert n > 4_000_000_000
    assert bad == 0 and out.returncode == 0
