"""Benchmark: cell-updates/s per RK3 step of the 3D Taylor-Green vortex at 256^3 with WENO5-JS
characteristic fluxes (Roe average, LLF splitting, eps = 1e-6), 4th-order central viscous terms,
Minf = 1.25, Re = 1600, dt fixed from CFL 0.5 on the initial state.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 256]

Own arm (default): the FP32-mixed path (FP32 state and flux arithmetic, FP64 RK accumulator) is
the headline `value`; the plain FP64 GPU path is timed beside it ("fp64"), and the mixed result's
L2 / Linf error against the FP64 run after the same steps is reported.  Inputs are device
resident (the state is 335 MB in FP32 and 2.7 GB with the FP64 register, both larger than the
129 MB L2).  `e2e` times the same step through the public API with the state uploaded from pinned
host memory before and read back after every step.  Replicas only: with N > 1 every rank runs its
own instance (one per GPU, no exchange) and value = total cell-updates / max time.

Reference arm (--impl reference): the reference generator's own C output for this problem
(oracle/_ref/tgv_weno, compiled with the OPS-API stand-in and OpenMP on all host cores), timed by
its own "Total Wall time" over K steps after a W-step warm-up run.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-updates/s per RK3 step"
UNIT = "cell-updates/s"
# algorithmic bytes per cell per RK stage (read+write of the state and of the RK register)
ALG_BYTES_STAGE = {"mixed": 5 * (2 * 4 + 2 * 8), "fp64": 5 * (2 * 8 + 2 * 8)}


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------------
# reference arm
# ------------------------------------------------------------------------------------------------
def reference_cpu(n, steps, warmup, dt, Minf, threads=None, allow_port=True):
    """Time the reference's generated C for the WENO TGV (or, if its generated sources are absent,
    the oracle's C restatement) on the host cores.  Returns a dict with cell-updates/s."""
    from oracle import refrun
    threads = threads or os.cpu_count()
    case = "tgv_weno"
    if refrun.available(case):
        refrun.build(case)
        params = dict(block0np0=n, block0np1=n, block0np2=n, dt=dt, Minf=Minf)
        import tempfile
        tmp = tempfile.mkdtemp(prefix="osb_bench_ref_")
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        for k, v in params.items():
            env["OSB_" + k] = repr(v) if isinstance(v, float) else str(v)
        exe = refrun.build(case)

        def run(niter):
            env["OSB_niter"] = str(niter)
            out = subprocess.run([exe], env=env, cwd=tmp, capture_output=True, text=True, timeout=3600)
            if out.returncode != 0:
                raise RuntimeError(out.stderr[-2000:])
            for line in out.stdout.splitlines():
                if "Total Wall time" in line:
                    return float(line.split()[-1])
            raise RuntimeError("no wall time in reference output")

        if warmup > 0:
            run(warmup)
        wall = run(steps)
        return {"value": n ** 3 * steps / wall, "wall_s": wall, "kind": "reference", "cores": threads,
                "sample": "reference generator's C for the WENO5-JS TGV (opensbli.cpp from LLFWeno(5,'JS'), "
                          "compiled with the OPS-API stand-in, OpenMP), %d^3, %d timed RK3 steps after a "
                          "%d-step warm-up run" % (n, steps, warmup)}
    if not allow_port:
        raise RuntimeError("reference sources not present")
    from oracle import oracle as O
    import math
    cfg = O.make_cfg((n, n, n), (2 * math.pi / n,) * 3, Minf=Minf, conv="weno5js", dt=dt)
    q0 = O.tgv_init(cfg)
    t0 = time.perf_counter()
    O.run(cfg, q0, steps)
    wall = time.perf_counter() - t0
    return {"value": n ** 3 * steps / wall, "wall_s": wall, "kind": "port", "cores": 1,
            "sample": "oracle C restatement (single thread), %d^3, %d RK3 steps" % (n, steps)}


def ref_arm(args, world, rank):
    if rank != 0:
        return
    from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt
    plan = tgv_plan(args.n, conv="weno5js", Minf=1.25)
    dt = tgv_cfl_dt(plan)
    # a bounded sample: the full grid, a few steps (each 256^3 WENO step takes seconds on the host)
    steps = max(1, min(args.steps, args.ref_steps))
    warm = max(0, min(args.warmup, 1))
    r = reference_cpu(args.n, steps, warm, dt, 1.25)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * r["wall_s"] / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: analytic Taylor-Green initial condition",
            "config": config_block(args.n, dt, "fp64"), "impl": "reference",
            "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"]},
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def config_block(n, dt, precision):
    return {"workload": "Taylor-Green vortex %d^3, WENO5-JS characteristic fluxes (Roe, LLF, eps=1e-6) + "
                        "4th-order central viscous terms, RK3 (2-register), Minf=1.25, Re=1600, Pr=0.71, "
                        "dt from CFL 0.5 on the initial state" % n,
            "grid": [n, n, n], "dt": dt, "precision": precision,
            "l2": "inputs larger than L2 (state %.0f MB FP32 + %.0f MB FP64 register)" % (
                5 * n ** 3 * 4 / 1e6, 5 * n ** 3 * 8 / 1e6)}


# ------------------------------------------------------------------------------------------------
# own arm
# ------------------------------------------------------------------------------------------------
def time_steps(solver, steps, dt, torch):
    st = solver.stream
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    solver.step(steps, dt)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def own_arm(args, world, rank, local):
    import numpy as np
    import torch
    from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt
    from opensbli_gb300.runtime import Solver

    torch.cuda.set_device(local)
    n = args.n
    plan = tgv_plan(n, conv="weno5js", Minf=1.25, precision="mixed")
    dt = tgv_cfl_dt(plan)
    cells = n ** 3
    K, W = args.steps, args.warmup

    # ---- mixed path: device-resident timing
    s = Solver(plan)
    s.init_tgv()
    s.step(W, dt)
    barrier(world)
    with ClockSampler(local) as clk:
        t = time_steps(s, K, dt, torch)
    launches = s.launch_count()
    t = max_over_ranks(t, world)
    value = world * cells * K / t
    q_mixed = s.state64()

    # ---- per-kernel-family timing (eager launches bracketed by CUDA events on the solver stream)
    s.profile(True)
    s.step(max(2, min(K, 5)), dt)
    torch.cuda.synchronize()
    prof = s.profile_read()
    s.profile(False)

    # ---- e2e through the public API: pinned host state in, host state out, every step
    s.init_tgv()
    host_in = s.state64().cpu().pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    e2e_steps = max(1, min(K, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dev = host_in.to(s.device, non_blocking=True)
        s.set_state64(dev)
        s.step(1, dt)
        host_out.copy_(s.state64(), non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = world * cells * e2e_steps / t_e2e
    bytes_io = 5 * cells * 8
    s.close()
    del s

    # ---- FP64 path on the same workload and error of the mixed run against it
    K64 = max(1, min(K, args.fp64_steps))
    s64 = Solver(plan.replace(precision="fp64"))
    s64.init_tgv()
    s64.step(min(W, 1), dt)
    t64 = time_steps(s64, K64, dt, torch)
    # FP64 reference state after W+K steps for the error of the mixed run
    s64.init_tgv()
    s64.step(W + K, dt)
    q64 = s64.state64()
    s64.close()
    del s64
    diff = (q_mixed - q64)
    l2 = [float(torch.linalg.vector_norm(diff[v]) / torch.linalg.vector_norm(q64[v])) for v in range(5)]
    linf = [float(diff[v].abs().max() / q64[v].abs().max()) for v in range(5)]

    # ---- roofline of the whole RK3 step and of the dominant kernel family
    peak, peak_kind = load_peaks()
    t_step = t / K
    achieved_step = cells * 3 * ALG_BYTES_STAGE["mixed"] / t_step / 1e9
    fam_bytes = {"weno_x": 5 * 4 * 2, "weno_y": 5 * 4 * 3, "weno_z": 5 * 4 * 3, "central_rk": 5 * (4 + 4 + 8 + 8 + 4),
                 "halo": 0}
    dom = max((f for f in prof if f in fam_bytes and fam_bytes[f] > 0), key=lambda f: prof[f][0], default=None)
    roof = None
    if dom:
        ms, cnt = prof[dom]
        per_launch = ms / cnt / 1e3
        ach = cells * fam_bytes[dom] / per_launch / 1e9
        roof = {"bound": "hbm", "kernel": "k_weno<float,%d>" % "xyz".index(dom[-1]) if dom.startswith("weno") else dom,
                "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_kind": peak_kind,
                "traffic": None, "alg_bytes_per_cell": fam_bytes[dom],
                "avg_launch_ms": per_launch * 1e3,
                "step": {"achieved": achieved_step, "frac": achieved_step / peak,
                         "alg_bytes_per_cell_per_stage": ALG_BYTES_STAGE["mixed"]}}
        steps_prof = max(2, min(K, 5))
        roof["families_ms_per_step"] = {f: prof[f][0] / steps_prof for f in prof}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            r = reference_cpu(n, args.ref_steps, 0, dt, 1.25)
            cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]}
        except Exception as e:
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "unavailable", "sample": str(e)[:200]}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": 1e3 * t / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (RK accumulator f64)", "data": "synthetic: analytic Taylor-Green initial condition",
                "config": dict(config_block(n, dt, "mixed"), parallelism="replicas" if world > 1 else "single"),
                "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_io,
                        "d2h_bytes_per_step": bytes_io, "steps": e2e_steps,
                        "path": "Solver.set_state64 (pinned host -> device) + Solver.step(1) + state64 -> pinned host"},
                "gpu_launches": launches, "clocks": clk.summary(),
                "fp64": {"value": world * cells * K64 / t64, "ms_per_step": 1e3 * t64 / K64, "steps": K64,
                         "mixed_speedup": (value / world) / (cells * K64 / t64)},
                "error_vs_fp64": {"steps": W + K, "l2": l2, "linf": linf,
                                  "vars": ["rho", "rhou0", "rhou1", "rhou2", "rhoE"]}}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--ref-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        ref_arm(args, world, rank)
    else:
        own_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
