"""A minimal driver for profiling one configuration (e.g. under ncu): initialise, run, synchronise.

    python -m opensbli_gb300.profile_case --n 192 --conv weno5js --precision mixed --steps 1 [--no-graphs]
        [--shape 1:march4:48 --shape 2:march4:48] [--central-ty 16]

Runs the Taylor-Green vortex with the given scheme and precision for --steps RK3 steps after
--warmup steps and prints the wall time per step (not a benchmark number: bench.py is).
"""
import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--conv", default="weno5js", choices=["weno5js", "weno5z", "teno5", "teno6", "central_skew"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--no-graphs", action="store_true")
    ap.add_argument("--shape", action="append", default=[],
                    help="dir:kind:seg launch shape of a WENO flux kernel (kind tile|march4|march8)")
    ap.add_argument("--central-ty", type=int, default=0, help="tile height of the central/RK kernel (8 or 16)")
    a = ap.parse_args()
    import torch
    from .plan import tgv_plan, tgv_cfl_dt
    from .runtime import Solver
    M = 0.1 if a.conv == "central_skew" else 1.25
    plan = tgv_plan(a.n, conv=a.conv, Minf=M, precision=a.precision, use_graphs=not a.no_graphs)
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
    print("n=%d conv=%s precision=%s: %.3f ms/step, launches %d, ke %.10f" % (
        a.n, a.conv, a.precision, 1e3 * dtw, s.launch_count(), s.reduce("ke")))
    s.close()


if __name__ == "__main__":
    main()
