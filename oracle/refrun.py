"""Build and run the reference generator's own C output (test infrastructure only).

oracle/gen/generate.py writes the generated sources of each case into oracle/_ref/<case>/ (this
needs the reference tree and runs only where it is present).  build(case) compiles them against
the OPS stand-in in oracle/ops_compat with g++ and OpenMP; run(case, ...) executes the binary with
run-time parameters (grid size, dt, step count) and reads back the conserved fields it dumps.
"""
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")


def case_dir(case):
    return os.path.join(REF, case)


def available(case):
    return os.path.exists(os.path.join(case_dir(case), "opensbli.cpp"))


def build(case, force=False):
    d = case_dir(case)
    src = os.path.join(d, "opensbli.cpp")
    exe = os.path.join(d, "ref_bin")
    deps = [src] + [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".h")]
    deps += [os.path.join(HERE, "ops_compat", f) for f in os.listdir(os.path.join(HERE, "ops_compat"))]
    if not force and os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(f) for f in deps):
        return exe
    subprocess.check_call(["g++", "-O2", "-fopenmp", "-I", os.path.join(HERE, "ops_compat"), "-I", d, src, "-o", exe])
    return exe


def load_dump(path, interior=True):
    hdr = np.fromfile(path, dtype=np.int32, count=12)
    size, dm, dp = hdr[1:4], hdr[4:7], hdr[7:10]
    pad = size - dm + dp
    a = np.fromfile(path, dtype=np.float64, offset=48).reshape(pad[2], pad[1], pad[0])
    if not interior:
        return a[0] if size[2] == 1 and pad[2] == 1 else a
    a = a[-dm[2]:-dm[2] + size[2], -dm[1]:-dm[1] + size[1], -dm[0]:-dm[0] + size[0]]
    return a[0] if size[2] == 1 and pad[2] == 1 else a


def run(case, params, variables, threads=None, outdir=None, timeout=3600):
    """Run the compiled case.  params: {name: value} for OSB_<name>; returns ({var: array}, wall_s)."""
    exe = build(case)
    env = dict(os.environ)
    for k, v in params.items():
        env["OSB_" + k] = repr(v) if isinstance(v, float) else str(v)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    tmp = outdir or tempfile.mkdtemp(prefix="osbref_")
    os.makedirs(tmp, exist_ok=True)
    env["OSB_DUMP_DIR"] = tmp
    out = subprocess.run([exe], env=env, cwd=tmp, capture_output=True, text=True, timeout=timeout)
    if out.returncode != 0:
        raise RuntimeError("reference binary failed: %s" % out.stderr[-2000:])
    m = re.search(r"Total Wall time ([0-9.eE+-]+)", out.stdout)
    wall = float(m.group(1)) if m else float("nan")
    fields = {v: load_dump(os.path.join(tmp, "opensbli_output.%s_B0.bin" % v)) for v in variables}
    return fields, wall
