"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Needs the reference tree ($OPENSBLI_REFERENCE, else ../reference beside the repository) and g++; run from the repository root:

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

sys.path.insert(0, os.path.join(REPO, "oracle", "gen"))
from refpath import default_ref  # noqa: E402

VARS = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]

# case -> (grid points per axis, steps, run-time parameter overrides)
CASES = {
    "tgv_central": (16, 20, {"dt": 5e-3}),
    "tgv_weno": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
    "tgv_wenoz": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
    "tgv_teno": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
    "tgv_teno6": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
    "tgsym_central": (17, 10, {"dt": 5e-3}),
    # central skew-symmetric scheme with the WENO5 non-linear filter (constant sensor) after every step
    "tgv_filter": (16, 10, {"dt": 3e-3, "Minf": 1.25}),
    # TENO5 with the cut-off adapted by the modified Ducros sensor
    "tgv_teno_adaptive": (16, 10, {"dt": 2e-3, "Minf": 1.25}),
}


# 2D case: grid (n0, n1), steps, overrides.  The fixture keeps the reference's initial state and
# final state with a 4-point halo (its initialisation kernel fills halos that the inlet reads) and
# the x1 coordinate the metrics are computed from.
CASES_2D = {
    "katzer_teno": ((64, 32), 20, {"dt": 0.01}),
    # the published script: TENO cut-off adapted by the modified Ducros sensor
    "katzer_adaptive": ((64, 32), 20, {"dt": 0.01}),
    # Carpenter closures (the reference's default) on the outlet and the wall, ReducedAccess elsewhere
    "katzer_carpenter": ((64, 32), 20, {"dt": 0.01}),
    # the other characteristic schemes on the 2D block
    "katzer_weno": ((64, 32), 20, {"dt": 0.01}),
    "katzer_wenoz": ((64, 32), 20, {"dt": 0.01}),
    "katzer_teno6": ((64, 32), 20, {"dt": 0.01}),
    # the inviscid shock reflection (Euler, WENO5-Z with SimpleAverage, Dirichlet inlet, symmetry
    # face, the shock generator's Dirichlet top), dt at CFL ~0.4 so that the shock moves
    "shock_reflection": ((64, 32), 30, {"dt": 1.0}),
    # the doubly periodic Euler density wave (WENO5-Z, simple average, two-register RK3)
    "euler_wave": ((32, 24), 40, {"dt": 5e-3}),
    # the viscous shock tube: adiabatic walls on three faces, a symmetry face, constant mu, Cartesian
    "viscous_shock_tube": ((48, 24), 40, {"dt": 1e-3}),
    # the laminar channel: skew-symmetric central convection, walls on both x1 faces, forcing
    "laminar_channel": ((16, 32), 40, {"dt": 2e-3}),
}
VARS_2D = ["rho", "rhou0", "rhou1", "rhoE"]

# 1D Euler case: n0, steps, overrides; the fixture keeps the initial and final states with a 4-point halo
CASES_1D = {
    "sod": (200, 200, {"dt": 2e-4}),
    "shu_osher": (400, 200, {"dt": 2e-3}),
}
VARS_1D = ["rho", "rhou0", "rhoE"]

# span-periodic 3D wall-bounded case: grid (n0, n1, n2), steps, overrides.  The fixture keeps the
# reference's initial and final states with a 4-point halo and the x1 coordinate line (x1 depends on
# j alone) with a 4-point halo.
CASES_3W = {
    "sbli3d_teno": ((32, 24, 8), 10, {"dt": 0.02}),
    # the transitional_SBLI block: adaptive TENO6 with the metric sensor, body force, Dirichlet face
    # with the spanwise kinetic energy
    # (forcing centred on a grid point of this coarse grid and 20x stronger, so that it shows)
    "transitional_sbli": ((32, 24, 8), 20, {"dt": 0.2, "A": 0.05, "xF": 2 * 375.0 / 31}),
    # the compressible_TCF_TENO channel block (statistics off) at the script's dt
    "channel_teno": ((32, 24, 16), 40, {"dt": 2e-4}),
}
VARS_3W = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]


def padded4(d, names):
    # dumps carry a 5-point halo; keep 4
    return {v: refrun.load_dump(os.path.join(d, "opensbli_output.%s_B0.bin" % v), interior=False)[1:-1, 1:-1]
            for v in names}


def main2d(ref, only=None):
    import tempfile
    for case, ((n0, n1), steps, extra) in CASES_2D.items():
        if only is not None and case != only:
            continue
        if not refrun.available(case):
            subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "generate.py"), "--case", case,
                                   "--ref", ref])
        base = dict(block0np0=n0, block0np1=n1)
        base.update(extra)
        d0 = tempfile.mkdtemp(prefix="osb_g0_")
        refrun.run(case, dict(base, niter=0), VARS_2D + ["x1"], threads=4, outdir=d0)
        ic = padded4(d0, VARS_2D + ["x1"])
        d1 = tempfile.mkdtemp(prefix="osb_g1_")
        refrun.run(case, dict(base, niter=steps), VARS_2D, threads=4, outdir=d1)
        fin = padded4(d1, VARS_2D)
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % case), q0=np.stack([ic[v] for v in VARS_2D]),
                            x1=ic["x1"], q=np.stack([fin[v] for v in VARS_2D]), n=np.array([n0, n1]), steps=steps,
                            params=json.dumps(dict(base, niter=steps)))
        out = os.path.join("/tmp", "osb_lower_%s" % case)
        subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", case,
                               "--out", out, "--ref", ref], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        with open(os.path.join(out, "plan.json")) as f:
            plan = json.load(f)
        with open(os.path.join(HERE, "plan_%s.json" % case), "w") as f:
            json.dump(plan, f, indent=1)
        print("wrote", case, fin["rho"].shape)


def main1d(ref, only=None):
    import tempfile
    for case, (n0, steps, extra) in CASES_1D.items():
        if only is not None and case != only:
            continue
        if not refrun.available(case):
            subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "generate.py"), "--case", case,
                                   "--ref", ref])
        base = dict(block0np0=n0)
        base.update(extra)
        d0 = tempfile.mkdtemp(prefix="osb_g0_")
        refrun.run(case, dict(base, niter=0), VARS_1D, threads=2, outdir=d0)
        ic = {v: refrun.load_dump(os.path.join(d0, "opensbli_output.%s_B0.bin" % v), interior=False).reshape(-1)[1:-1]
              for v in VARS_1D}
        d1 = tempfile.mkdtemp(prefix="osb_g1_")
        refrun.run(case, dict(base, niter=steps), VARS_1D, threads=2, outdir=d1)
        fin = {v: refrun.load_dump(os.path.join(d1, "opensbli_output.%s_B0.bin" % v), interior=False).reshape(-1)[1:-1]
               for v in VARS_1D}
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % case), q0=np.stack([ic[v] for v in VARS_1D]),
                            q=np.stack([fin[v] for v in VARS_1D]), n=np.array([n0]), steps=steps,
                            params=json.dumps(dict(base, niter=steps)))
        out = os.path.join("/tmp", "osb_lower_%s" % case)
        r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", case,
                            "--out", out, "--ref", ref], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode == 0:
            with open(os.path.join(out, "plan.json")) as f:
                plan = json.load(f)
            with open(os.path.join(HERE, "plan_%s.json" % case), "w") as f:
                json.dump(plan, f, indent=1)
        print("wrote", case, fin["rho"].shape, "plan" if r.returncode == 0 else "(no plan: lowering failed)")


def main3w(ref, only=None):
    import tempfile
    for case, ((n0, n1, n2), steps, extra) in CASES_3W.items():
        if only is not None and case != only:
            continue
        if not refrun.available(case):
            subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "generate.py"), "--case", case,
                                   "--ref", ref])
        base = dict(block0np0=n0, block0np1=n1, block0np2=n2)
        base.update(extra)
        d0 = tempfile.mkdtemp(prefix="osb_g0_")
        refrun.run(case, dict(base, niter=0), VARS_3W + ["x1"], threads=4, outdir=d0)
        ic = {v: refrun.load_dump(os.path.join(d0, "opensbli_output.%s_B0.bin" % v), interior=False)[1:-1, 1:-1, 1:-1]
              for v in VARS_3W + ["x1"]}
        d1 = tempfile.mkdtemp(prefix="osb_g1_")
        refrun.run(case, dict(base, niter=steps), VARS_3W, threads=4, outdir=d1)
        fin = {v: refrun.load_dump(os.path.join(d1, "opensbli_output.%s_B0.bin" % v), interior=False)[1:-1, 1:-1, 1:-1]
               for v in VARS_3W}
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % case), q0=np.stack([ic[v] for v in VARS_3W]),
                            x1=ic["x1"][4, :, 4], q=np.stack([fin[v] for v in VARS_3W]), n=np.array([n0, n1, n2]),
                            steps=steps, params=json.dumps(dict(base, niter=steps)))
        out = os.path.join("/tmp", "osb_lower_%s" % case)
        r = subprocess.run([sys.executable, os.path.join(REPO, "oracle", "gen", "lower_case.py"), "--case", case,
                            "--out", out, "--ref", ref], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        if r.returncode == 0:
            with open(os.path.join(out, "plan.json")) as f:
                plan = json.load(f)
            with open(os.path.join(HERE, "plan_%s.json" % case), "w") as f:
                json.dump(plan, f, indent=1)
        print("wrote", case, fin["rho"].shape, "plan" if r.returncode == 0 else "(no plan: lowering failed)")


def main(ref=None, only=None):
    """Regenerate every fixture, or only the case `only`."""
    ref = ref or default_ref()
    if only is None:
        main1d(ref)
        main2d(ref)
        main3w(ref)
        katzer_profile(ref)
    elif only in CASES_2D:
        main2d(ref, only)
        return
    elif only in CASES_3W:
        main3w(ref, only)
        return
    elif only in CASES_1D:
        main1d(ref, only)
        return
    for case, (n, steps, extra) in CASES.items():
        if only is not None and case != only:
            continue
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


def katzer_profile(ref=None, n1=256, n0=512):
    """The reference's Katzer initial state on n1 = 256 rows (it is independent of x0): one padded
    column of rho, rhou0, rhou1, rhoE and x1 with a 4-point halo, for the 512 x 256 benchmark."""
    import tempfile
    ref = ref or default_ref()
    case = "katzer_teno"
    if not refrun.available(case):
        subprocess.check_call([sys.executable, os.path.join(REPO, "oracle", "gen", "generate.py"), "--case", case,
                               "--ref", ref])
    d = tempfile.mkdtemp(prefix="osb_kic_")
    refrun.run(case, dict(block0np0=n0, block0np1=n1, niter=0), VARS_2D + ["x1"], threads=8, outdir=d)
    p = padded4(d, VARS_2D + ["x1"])
    np.savez_compressed(os.path.join(HERE, "katzer_ic_n%d.npz" % n1),
                        q_col=np.stack([p[v][:, 4] for v in VARS_2D]), x1_col=p["x1"][:, 4], n1=n1)


if __name__ == "__main__":
    main(*sys.argv[1:])
