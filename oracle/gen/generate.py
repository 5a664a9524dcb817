"""Run an OpenSBLI problem script through the reference generator and keep its C output.

Test infrastructure (oracle).  Usage, from the repository root:

    python oracle/gen/generate.py --case tgv_central [--ref REFERENCE_TREE] [--out oracle/_ref]

The reference generator (opensbli, read-only, imported from --ref) runs unmodified under the
compatibility shims in compat.py.  Its OPSC writer (code_generation/opsc.py:250-282) writes
opensbli.cpp, opensbliblock00_kernels.h, defdec_data_set.h and bc_exchanges.h into
<out>/<case>/.  The script's final substitute_simulation_parameters call
(utilities/helperfunctions.py:130-149) is replaced by one that writes every `X=Input;` as
`X = osb_param_i/d("X", <script value>);`, so one compiled binary takes its grid size, dt and
step count from OSB_<X> environment variables at run time (ops_compat/ops_seq.h).
"""
import argparse
import os
import re
import runpy
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

# case name -> problem script.  "ref:" paths are inside the reference tree, others under cases/.
CASES = {
    "tgv_central": "ref:apps/taylor_green_vortex/taylor_green_vortex.py",
    "tgsym_central": "ref:apps/taylor_green_vortex/TGsym/TGsym.py",
    "tgv_weno": "tgv_weno.py",
    "tgv_wenoz": "tgv_wenoz.py",
    "tgv_teno": "tgv_teno.py",
    "tgv_teno6": "tgv_teno6.py",
    "tgv_filter": "tgv_filter.py",
    "tgv_teno_adaptive": "tgv_teno_adaptive.py",
    "tgv_weno_modified": "tgv_weno_modified.py",
    "katzer_teno": "katzer_teno.py",
    "katzer_carpenter": "katzer_carpenter.py",
    "katzer_weno": "katzer_weno.py",
    "katzer_wenoz": "katzer_wenoz.py",
    "katzer_teno6": "katzer_teno6.py",
    "katzer_adaptive": "ref:apps/katzer_SBLI/katzer_SBLI.py",
    "sbli3d_teno": "sbli3d_teno.py",
    "transitional_sbli": "transitional_sbli.py",
    "channel_teno": "channel_teno.py",
    "shock_reflection": "ref:apps/inviscid_shock_reflection/inviscid_shock.py",
    "sod": "ref:apps/Sod_shock_tube/Sod_shock_tube.py",
    "shu_osher": "ref:apps/shu_osher/shu_osher.py",
    "euler_wave": "ref:apps/euler_wave/euler_wave.py",
    "kelvin_helmholtz": "ref:apps/kelvin_helmholtz/kelvin_helmholtz.py",
    "viscous_shock_tube": "ref:apps/viscous_shock_tube/viscous_shock_tube.py",
    "laminar_channel": "ref:apps/channel_flow/laminar_2D/laminar_channel.py",
}


def _runtime_substitution(constants, values, simulation_name="opensbli"):
    path = "./%s.cpp" % simulation_name
    with open(path) as f:
        s = f.read()
    for const, value in zip(constants, values):
        old = const + "=Input;"
        if old not in s:
            continue
        is_int = re.search(r"^int %s;" % re.escape(const), s, re.M) is not None
        fn = "osb_param_i" if is_int else "osb_param_d"
        s = s.replace(old, '%s = %s("%s", %s);' % (const, fn, const, value))
    left = re.findall(r"(\w+)=Input;", s)
    if left:
        raise RuntimeError("constants left without a value: %s" % left)
    with open(path, "w") as f:
        f.write(s)


def run_case_inproc(case, ref):
    sys.path.insert(0, HERE)
    sys.path.insert(0, ref)
    import compat
    compat.install()
    import opensbli.utilities.helperfunctions as hf
    hf.substitute_simulation_parameters = _runtime_substitution
    script = CASES[case]
    if script.startswith("ref:"):
        script = os.path.join(ref, script[4:])
    else:
        script = os.path.join(HERE, "cases", script)
    runpy.run_path(script, run_name="__main__")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True, choices=sorted(CASES) + ["all"])
    from refpath import default_ref
    ap.add_argument("--ref", default=default_ref(),
                    help="reference tree (default: $OPENSBLI_REFERENCE, else ../reference beside the repository)")
    ap.add_argument("--out", default=os.path.join(REPO, "oracle", "_ref"))
    ap.add_argument("--inproc", action="store_true", help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.inproc:
        run_case_inproc(a.case, a.ref)
        return
    cases = sorted(CASES) if a.case == "all" else [a.case]
    for case in cases:
        out = os.path.join(os.path.abspath(a.out), case)
        os.makedirs(out, exist_ok=True)
        log = os.path.join(out, "generate.log")
        with open(log, "w") as lf:
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--case", case, "--ref", a.ref, "--inproc"],
                               cwd=out, stdout=lf, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            sys.stderr.write(open(log).read()[-4000:])
            raise SystemExit("generation of %s failed (log: %s)" % (case, log))
        print("generated %s -> %s" % (case, out))


if __name__ == "__main__":
    main()
