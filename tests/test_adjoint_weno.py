"""The reverse mode of the FP64 characteristic interface flux used by the adjoint of WENO5-JS,
WENO5-Z, TENO5 and TENO6 plans (opensbli_gb300/csrc/osb_adjoint_weno.cuh), compiled for the host with
g++ and checked against central finite differences of its own forward flux in all three directions
(tests/native/adjw_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "opensbli_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_interface_flux_reverse_mode_matches_finite_differences(tmp_path):
    exe = str(tmp_path / "adjw_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "adjw_check.cpp"),
                           "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    lines = out.stdout.split("\n")
    assert out.returncode == 0 and lines[4] == "windows 3600"
    worst = {int(l.split()[0]): float(l.split()[1]) for l in lines[:4]}
    assert max(worst.values()) < 1e-6, worst  # WENO5-JS, WENO5-Z, TENO5, TENO6
