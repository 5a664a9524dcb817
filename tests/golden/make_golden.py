"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Needs the reference tree (default /root/reference) and g++; run from the repository root:

    python tests/golden/make_golden.py

For every case it (1) runs the reference generator on the case's problem script
(oracle/gen/generate.py), (2) compiles the generated C against the OPS stand-in and runs it at a
small size (oracle/refrun.py), and stores the conserved fields after the stated number of steps as
ref_<case>.npz; (3) lowers the same script with GB300Writer (oracle/gen/lower_case.py) and stores
the Plan as plan_<case>.json.  The fixtures are what the CPU tests pin the oracle against and
what the GPU tests compare with where the reference is not installed.
"""
import json
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import refrun  # noqa: E402

VARS = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]

# case -> (grid points per axis, steps, run-time parameter overrides)
CASES = {
    "tgv_central": (16, 20, {"dt": 5e-3}),
    "tgv_weno": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
    "tgsym_central": (17, 10, {"dt": 5e-3}),
}


def main(ref="/root/reference"):
    for case, (n, steps, extra) in CASES.items():
        if not refrun.available(case):
            subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "generate.py"), "--case", case,
                                   "--ref", ref])
        params = dict(block0np0=n, block0np1=n, block0np2=n, niter=steps)
        params.update(extra)
        fields, _ = refrun.run(case, params, VARS, threads=4)
        q = np.stack([fields[v] for v in VARS])
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % case), q=q, n=n, steps=steps,
                            params=json.dumps(params))
        out = os.path.join("/tmp", "osb_lower_%s" % case)
        subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", case,
                               "--out", out, "--ref", ref], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        with open(os.path.join(out, "plan.json")) as f:
            plan = json.load(f)
        with open(os.path.join(HERE, "plan_%s.json" % case), "w") as f:
            json.dump(plan, f, indent=1)
        print("wrote", case, q.shape)


if __name__ == "__main__":
    main(*sys.argv[1:])
