"""A minimal driver for profiling one configuration (e.g. under ncu): initialise, run, synchronise.

    python -m opensbli_gb300.profile_case --n 192 --conv weno5js --precision mixed --steps 1 [--no-graphs]
        [--shape 1:march4:48 --shape 2:march4:48] [--central-ty 16] [--adaptive] [--filter]
    python -m opensbli_gb300.profile_case --katzer 512 [--conv teno5|teno6|weno5js|weno5z] [--adaptive]

Runs the Taylor-Green vortex (or, with --katzer N0, the 2D shock/boundary-layer block N0 x 256 from
the boundary-layer profile in tests/golden/katzer_ic_n256.npz) with the given scheme and precision
for --steps RK3 steps after --warmup steps and prints the wall time per step (not a benchmark
number: bench.py is).
"""
import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--conv", default=None, choices=["weno5js", "weno5z", "teno5", "teno6", "central_skew"],
                    help="default weno5js (Taylor-Green), teno5 (--katzer)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--no-graphs", action="store_true")
    ap.add_argument("--shape", action="append", default=[],
                    help="dir:kind:seg launch shape of a WENO flux kernel (kind tile|march4|march8)")
    ap.add_argument("--central-ty", type=int, default=0, help="tile height of the central/RK kernel (8 or 16)")
    ap.add_argument("--adaptive", action="store_true", help="TENO cut-off adapted by the modified Ducros sensor")
    ap.add_argument("--filter", action="store_true", help="WENO5 non-linear filter after every step")
    ap.add_argument("--katzer", type=int, default=0, help="2D shock/boundary-layer block of this many x0 points")
    a = ap.parse_args()
    import torch
    from .plan import tgv_plan, tgv_cfl_dt
    from .runtime import Solver
    if a.katzer:
        import os
        import numpy as np
        from .plan import katzer_plan
        n0, n1 = a.katzer, 256
        a.conv = a.conv or "teno5"
        plan = katzer_plan(n0, n1, precision=a.precision, conv=a.conv, dt=0.04, use_graphs=not a.no_graphs,
                           adaptive=a.adaptive)
        dt = 0.04
        ic = np.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                                  "katzer_ic_n%d.npz" % n1))
        s = Solver(plan)
        s.set_coordinate(np.repeat(ic["x1_col"][:, None], n0 + 8, axis=1), 4)
        s.set_state64_padded(np.repeat(ic["q_col"][:, :, None], n0 + 8, axis=2), 4)
        a.n = n0
    else:
        a.conv = a.conv or "weno5js"
        M = 0.1 if a.conv == "central_skew" else 1.25
        plan = tgv_plan(a.n, conv=a.conv, Minf=M, precision=a.precision, use_graphs=not a.no_graphs)
        plan = plan.replace(teno_adaptive=a.adaptive, filter="weno5_constant" if a.filter else "none")
        dt = tgv_cfl_dt(plan)
        s = Solver(plan)
        s.init_tgv()
    if a.central_ty:
        s.set_central_shape(a.central_ty)
    for sh in a.shape:
        d, kind, seg = sh.split(":")
        s.set_weno_shape(int(d), kind, int(seg))
    s.step(a.warmup, dt) if a.warmup else None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.step(a.steps, dt)
    torch.cuda.synchronize()
    dtw = (time.perf_counter() - t0) / max(a.steps, 1)
    print("n=%d conv=%s%s%s precision=%s: %.3f ms/step, launches %d, ke %.10f" % (
        a.n, a.conv, " adaptive" if a.adaptive else "", " filter" if a.filter else "", a.precision, 1e3 * dtw,
        s.launch_count(), s.reduce("ke") if plan.ndim == 3 else float("nan")))
    s.close()


if __name__ == "__main__":
    main()
