"""Lower a reference problem script with GB300Writer (test infrastructure).

    python oracle/gen/lower_case.py --case tgv_central --out DIR [--ref REFERENCE_TREE]

Runs the case's problem script in this process with the reference generator imported from --ref
(shims from compat.py), lets its OPSC call run as usual, hands the algorithm to
opensbli_gb300.GB300Writer, applies the script's own substitute_simulation_parameters values, and
writes DIR/plan.json (the lowered Plan) and DIR/ic.npy (the FP64 initial state evaluated from the
script's initialisation kernel).  Used by the CPU tests of the writer and by the fixture script.
"""
import argparse
import json
import os
import runpy
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def lower(case, ref, out, n=None, params=None):
    sys.path.insert(0, HERE)
    sys.path.insert(0, ref)
    sys.path.insert(0, REPO)
    import compat
    compat.install()
    import numpy as np
    import opensbli.utilities.helperfunctions as hf
    from generate import CASES
    from opensbli_gb300.writer import GB300Writer

    captured = {}
    import opensbli.code_generation.opsc as opsc_mod
    real_opsc = opsc_mod.OPSC

    class CapturingOPSC(real_opsc):
        def __init__(self, algorithm, *a, **k):
            captured["alg"] = algorithm
            real_opsc.__init__(self, algorithm, *a, **k)

    opsc_mod.OPSC = CapturingOPSC
    import opensbli
    import opensbli.code_generation as cg
    opensbli.OPSC = CapturingOPSC
    cg.OPSC = CapturingOPSC

    def subst(constants, values, simulation_name="opensbli"):
        captured["constants"] = (list(constants), list(values))

    hf.substitute_simulation_parameters = subst
    script = CASES[case]
    script = os.path.join(ref, script[4:]) if script.startswith("ref:") else os.path.join(HERE, "cases", script)
    os.makedirs(out, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(out)
    try:
        runpy.run_path(script, run_name="__main__")
    finally:
        os.chdir(cwd)
    w = GB300Writer(captured["alg"])
    consts, vals = captured["constants"]
    if n is not None:
        for d in range(3):
            if "block0np%d" % d in consts:
                vals[consts.index("block0np%d" % d)] = str(n if d == 0 else (n // 2 if w.plan.ndim == 2 else n))
    for k, v in (params or {}).items():
        vals[consts.index(k)] = v
    w.substitute_simulation_parameters(consts, vals)
    with open(os.path.join(out, "plan.json"), "w") as f:
        f.write(w.plan.to_json())
    if w.plan.ndim == 1:
        f = w.initial_fields(halo=4)
        np.save(os.path.join(out, "ic.npy"), np.stack([f[v] for v in w.state_names()]))
    elif w.plan.ndim == 2:
        f = w.initial_fields(halo=4)
        np.save(os.path.join(out, "ic.npy"), np.stack([f[v] for v in w.state_names()]))
        np.save(os.path.join(out, "x1.npy"), f["x1"])
    else:
        np.save(os.path.join(out, "ic.npy"), w.initial_state())
    with open(os.path.join(out, "constants.json"), "w") as f:
        json.dump({"constants": consts, "values": vals}, f)
    with open(os.path.join(out, "io.json"), "w") as f:
        json.dump(w.io_requests(), f)
    return w.plan


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True)
    ap.add_argument("--out", required=True)
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from refpath import default_ref
    ap.add_argument("--ref", default=default_ref())
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--params", default="", help="name=value,... overrides of the script's simulation parameters")
    a = ap.parse_args()
    p = lower(a.case, a.ref, a.out, a.n, dict(kv.split("=", 1) for kv in a.params.split(",") if kv))
    print(p.to_json())
