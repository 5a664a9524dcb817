"""A minimal driver for profiling one configuration (e.g. under ncu): initialise, run, synchronise.

    python -m opensbli_gb300.profile_case --n 192 --conv weno5js --precision mixed --steps 1 [--no-graphs]
        [--shape 1:march4:48 --shape 2:march4:48] [--central-ty 16] [--adaptive] [--filter]
    python -m opensbli_gb300.profile_case --katzer 512 [--conv teno5|teno6|weno5js|weno5z] [--adaptive]
    python -m opensbli_gb300.profile_case --sbli3d 256 --n2 64 [--conv ...]
    python -m opensbli_gb300.profile_case --channel 129 [--conv ...]
    python -m opensbli_gb300.profile_case --shock-reflection 457 [--conv ...]

Runs the Taylor-Green vortex (or, with --katzer N0, the 2D shock/boundary-layer block N0 x 256 from
the boundary-layer profile in tests/golden/katzer_ic_n256.npz, or with --sbli3d N0 the span-periodic
3D block N0 x 256 x n2 from the same profile with a spanwise momentum 0.05 sin(2 pi k / n2), or with
--channel N the N^3 channel block of compressible_TCF_TENO from its initial condition) with
the given scheme and precision
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
    ap.add_argument("--sbli3d", type=int, default=0, help="3D span-periodic block of this many x0 points")
    ap.add_argument("--n2", type=int, default=32, help="--sbli3d: points along the periodic x2 axis")
    ap.add_argument("--channel", type=int, default=0, help="the N^3 channel block (turbulent_channel.py)")
    ap.add_argument("--shock-reflection", type=int, default=0,
                    help="the 2D inviscid shock reflection of this many x0 points (inviscid_shock.py)")
    a = ap.parse_args()
    import torch
    from .plan import tgv_plan, tgv_cfl_dt
    from .runtime import Solver
    if a.shock_reflection:
        import numpy as np
        from .plan import shock_reflection_plan
        a.conv = a.conv or "weno5z"
        plan = shock_reflection_plan(a.shock_reflection, 255, precision=a.precision, conv=a.conv,
                                     use_graphs=not a.no_graphs)
        dt = plan.dt
        free = np.array(plan.dirichlet_x0[0])  # the free stream everywhere, as the script starts
        s = Solver(plan)
        s.set_state64_padded(np.ascontiguousarray(np.broadcast_to(free[:, None, None], (4, 255 + 8, plan.n[0] + 8))), 4)
        a.n = plan.n[0]
    elif a.channel:
        from .plan import channel_plan, channel_initial_state
        a.conv = a.conv or "teno6"
        plan = channel_plan(a.channel, a.channel, a.channel, precision=a.precision, conv=a.conv,
                            use_graphs=not a.no_graphs)
        dt = plan.dt
        q, x1 = channel_initial_state(plan, halo=3)
        s = Solver(plan)
        s.set_coordinate(x1, 3)
        s.set_state64_padded(q, 3)
        a.n = a.channel
    elif a.sbli3d:
        import os
        import numpy as np
        from .plan import sbli3d_plan
        n0, n1, n2 = a.sbli3d, 256, a.n2
        a.conv = a.conv or "teno5"
        plan = sbli3d_plan(n0, n1, n2, precision=a.precision, conv=a.conv, dt=0.04, use_graphs=not a.no_graphs)
        dt = 0.04
        ic = np.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                                  "katzer_ic_n%d.npz" % n1))
        col = ic["q_col"][:, 1:-1]  # 3-point halo in x1
        q = np.zeros((5, n2 + 6, n1 + 6, n0 + 6))
        w = 0.05 * np.sin(2 * np.pi * np.arange(-3, n2 + 3) / n2)
        for v, src in ((0, 0), (1, 1), (2, 2), (4, 3)):
            q[v] = col[src][None, :, None]
        q[3] = w[:, None, None] * np.ones((1, n1 + 6, n0 + 6))
        q[4] += 0.5 * q[3] ** 2 / q[0]
        s = Solver(plan)
        s.set_coordinate(ic["x1_col"], 4)
        s.set_state64_padded(q, 3)
        a.n = n0
    elif a.katzer:
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
