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

Other workloads (--config): tgv_central64 (the central Taylor-Green case), katzer512 and
katzer512_adaptive (the 2D shock/boundary-layer block), channel129 (the compressible_TCF_TENO channel,
129^3), shock_reflection (the 2D inviscid shock reflection, 457 x 255), tgv_adjoint128 (the discrete
adjoint) and tgv_batch96 (an ensemble of 96 blocks); each with the reference's generated C for the
same problem as its host-core arm where one exists.
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


# DRAM bytes per cell per launch measured by ncu for the mixed WENO TGV kernels at 192^3 (state larger
# than L2), used to scale the roofline's traffic figure to the benchmark's grid
DRAM_BYTES_PER_CELL_WENO_MIXED = {"weno_x": 46.0, "weno_y": 57.2, "weno_z": 57.4, "central_rk": 147.3}
# thread-instructions per cell (one interface per cell and direction) executed by the same kernels in
# the same capture (smsp__inst_executed x 32 / cells): the work that the FP32 issue rate bounds
THREAD_INST_PER_CELL_WENO_MIXED = {"weno_x": 1302.0, "weno_y": 1171.0, "weno_z": 1163.0}
SM_COUNT, SCHEDULERS_PER_SM, WARP = 152, 4, 32


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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


def dist_init(backend="nccl"):
    """One process per GPU (torchrun's RANK / WORLD_SIZE / LOCAL_RANK).  The ranks are independent
    replicas: the only collectives are the barrier around the timed region and the max of the times."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, steps, t_max, world):
    """Whole-job throughput of N replicas: every rank processes the same units per step; the job
    time is the slowest rank's."""
    return world * units_per_rank * steps / t_max


# ------------------------------------------------------------------------------------------------
# reference arm
# ------------------------------------------------------------------------------------------------
def reference_cpu(wl, steps, warmup, threads=None, allow_port=True):
    """Time the reference generator's C for the workload (or, if its generated sources are absent,
    the oracle's C restatement) on the host cores.  Returns a dict with cell-updates/s."""
    from oracle import refrun
    threads = threads or os.cpu_count()
    case = wl.cpu_case
    if refrun.available(case):
        import tempfile
        exe = refrun.build(case)
        tmp = tempfile.mkdtemp(prefix="osb_bench_ref_")
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        for k, v in wl.cpu_params.items():
            env["OSB_" + k] = repr(v) if isinstance(v, float) else str(v)

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
        return {"value": wl.cells * steps / wall, "wall_s": wall, "kind": "reference", "cores": threads,
                "sample": "the reference generator's C for this problem (oracle/_ref/%s: opensbli.cpp and kernels "
                          "from the reference's OPSC writer, compiled with the OPS-API stand-in and OpenMP), full "
                          "grid, %d timed RK3 steps after a %d-step warm-up run" % (case, steps, warmup)}
    if not allow_port or wl.plan.ndim != 3:
        raise RuntimeError("reference sources not present")
    from oracle import oracle as O
    p = wl.plan
    cfg = O.make_cfg(p.n, p.delta, Minf=p.Minf, conv=p.conv, dt=wl.dt)
    q0 = O.tgv_init(cfg)
    t0 = time.perf_counter()
    O.run(cfg, q0, steps)
    wall = time.perf_counter() - t0
    return {"value": wl.cells * steps / wall, "wall_s": wall, "kind": "port", "cores": 1,
            "sample": "oracle C restatement (single thread), full grid, %d RK3 steps" % steps}


def ref_arm(args, world, rank):
    if rank != 0:
        return
    wl = workload(args.config, args.n)
    steps = max(1, min(args.steps, args.ref_steps))
    warm = max(0, min(args.warmup, 1))
    r = reference_cpu(wl, steps, warm)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * r["wall_s"] / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: the problem's analytic initial condition",
            "config": dict(wl.config, precision="fp64"), "impl": "reference",
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


class Workload:
    """One benchmark configuration: how to build an initialised solver, its size and dt."""

    def __init__(self, name, plan, dt, init, config, cpu_case, cpu_params, alg_bytes):
        self.name, self.plan, self.dt, self.init = name, plan, dt, init
        self.config, self.cpu_case, self.cpu_params, self.alg_bytes = config, cpu_case, cpu_params, alg_bytes

    @property
    def cells(self):
        return self.plan.cells

    def solver(self, precision):
        """A solver holding the initial state, its kernel launch shapes autotuned on that state
        (untimed set-up)."""
        from opensbli_gb300.runtime import Solver
        s = Solver(self.plan.replace(precision=precision))
        self.init(s)
        s.autotune(reps=3)
        return s


def workload(name, n=None):
    import numpy as np
    from opensbli_gb300.plan import tgv_plan, tgv_cfl_dt, katzer_plan
    if name == "tgv_weno256":
        n = n or 256
        plan = tgv_plan(n, conv="weno5js", Minf=1.25)
        dt = tgv_cfl_dt(plan)
        return Workload(name, plan, dt, lambda s: s.init_tgv(), config_block(n, dt, "mixed"), "tgv_weno",
                        dict(block0np0=n, block0np1=n, block0np2=n, dt=dt, Minf=1.25),
                        {"mixed": 5 * (2 * 4 + 2 * 8), "fp64": 5 * (2 * 8 + 2 * 8)})
    if name == "tgv_central64":
        n = n or 64
        plan = tgv_plan(n, conv="central_skew", Minf=0.1)
        dt = 5e-3
        cfg = {"workload": "Taylor-Green vortex %d^3 on [0,2pi)^3, 4th-order central skew-symmetric convective and "
                           "viscous terms, RK3 (2-register), Minf=0.1, Re=1600, Pr=0.71, dt=5e-3" % n,
               "grid": [n, n, n], "dt": dt, "precision": "fp64",
               "l2": "inputs smaller than L2 (%.0f MB state); a step reads and writes every array" % (5 * n ** 3 * 8 / 1e6)}
        return Workload(name, plan, dt, lambda s: s.init_tgv(), cfg, "tgv_central",
                        dict(block0np0=n, block0np1=n, block0np2=n, dt=dt, Minf=0.1),
                        {"mixed": 5 * (2 * 4 + 2 * 8), "fp64": 5 * (2 * 8 + 2 * 8)})
    if name in ("katzer512", "katzer512_adaptive"):
        adaptive = name.endswith("_adaptive")
        n0, n1 = (n or 512), 256
        plan = katzer_plan(n0, n1, dt=0.04, adaptive=adaptive)
        d = np.load(os.path.join(REPO, "tests", "golden", "katzer_ic_n%d.npz" % n1))
        q = np.repeat(d["q_col"][:, :, None], n0 + 8, axis=2)
        x1 = np.repeat(d["x1_col"][:, None], n0 + 8, axis=1)

        def init(s):
            s.set_coordinate(x1, 4)
            s.set_state64_padded(q, 4)
        cut = ("C_T adapted per interface by the modified Ducros sensor (a1=10.5, a2=4.5)" if adaptive
               else "C_T=1e-5")
        cfg = {"workload": "2D shock/boundary-layer interaction %dx%d (Katzer): TENO5 (%s, eps=1e-15), "
                           "metrics stretched in x1 (sinh, factor 5), Sutherland viscosity, isothermal wall "
                           "Tw=1.676, shock-generator top face, LS-RK3 SSP, Mach 2, Re=950, dt=0.04" % (n0, n1, cut),
               "grid": [n0, n1], "dt": 0.04, "precision": "mixed",
               "l2": "inputs smaller than L2 (%.0f MB state)" % (4 * n0 * n1 * 8 / 1e6)}
        return Workload(name, plan, 0.04, init, cfg, "katzer_adaptive" if adaptive else "katzer_teno",
                        dict(block0np0=n0, block0np1=n1, dt=0.04),
                        {"mixed": 4 * (2 * 4 + 2 * 8) + 4, "fp64": 4 * (2 * 8 + 2 * 8) + 8})
    if name == "channel129":
        from opensbli_gb300.plan import channel_plan, channel_initial_state
        n = n or 129
        plan = channel_plan(n, n, n)
        q, x1 = channel_initial_state(plan, halo=3)

        def init(s):
            s.set_coordinate(x1, 3)
            s.set_state64_padded(q, 3)
        cfg = {"workload": "compressible turbulent channel %d^3 (compressible_TCF_TENO, statistics off): TENO6 "
                           "(C_T=1e-7), periodic x0/x2, isothermal walls on both x1 faces, x1 tanh-clustered (1.7), "
                           "mu=T^0.7, forcing c=(-1,0,0), LS-RK3 SSP, Re=190.71, Minf=0.0955, dt=2e-4" % n,
               "grid": [n, n, n], "dt": plan.dt, "precision": "mixed",
               "l2": "inputs larger than L2 (state %.0f MB FP32 + %.0f MB FP64 master and register)" %
                     (5 * n ** 3 * 4 / 1e6, 2 * 5 * n ** 3 * 8 / 1e6)}
        return Workload(name, plan, plan.dt, init, cfg, "channel_teno", dict(block0np0=n, block0np1=n, block0np2=n,
                        dt=plan.dt), {"mixed": 5 * (2 * 4 + 2 * 8), "fp64": 5 * (2 * 8 + 2 * 8)})
    if name == "shock_reflection":
        from opensbli_gb300.plan import shock_reflection_plan
        n0, n1 = (n or 457), 255
        plan = shock_reflection_plan(n0, n1)
        g = plan.gama
        free = np.array(plan.dirichlet_x0[0])
        q = np.ascontiguousarray(np.broadcast_to(free[:, None, None], (4, n1 + 8, n0 + 8)))
        cfg = {"workload": "2D inviscid shock reflection %dx%d (inviscid_shock.py): Euler, WENO5-Z with the simple "
                           "average, Dirichlet inlet, extrapolation, symmetry face, shock-generator top face, "
                           "LS-RK3, Mach 2, gama=%g, dt=0.1" % (n0, n1, g),
               "grid": [n0, n1], "dt": plan.dt, "precision": "mixed",
               "l2": "inputs smaller than L2 (%.0f MB state)" % (4 * n0 * n1 * 8 / 1e6)}
        return Workload(name, plan, plan.dt, lambda s: s.set_state64_padded(q, 4), cfg, "shock_reflection",
                        dict(block0np0=n0, block0np1=n1, dt=plan.dt),
                        {"mixed": 4 * (2 * 4 + 2 * 8), "fp64": 4 * (2 * 8 + 2 * 8)})
    raise SystemExit("unknown config %s" % name)


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
    import torch

    torch.cuda.set_device(local)
    wl = workload(args.config, args.n)
    dt, cells = wl.dt, wl.cells
    K, W = args.steps, args.warmup
    head = "mixed" if wl.config["precision"] == "mixed" else "fp64"
    other = "fp64" if head == "mixed" else "mixed"

    # ---- headline precision: device-resident timing
    s = wl.solver(head)
    s.step(W, dt)
    barrier(world)
    with ClockSampler(local) as clk:
        t = time_steps(s, K, dt, torch)
    launches = s.launch_count()
    t = max_over_ranks(t, world)
    value = aggregate_rate(cells, K, t, world)
    q_head = s.state64()

    # ---- per-kernel-family timing (eager launches bracketed by CUDA events on the solver stream)
    steps_prof = max(2, min(K, 5))
    s.profile(True)
    s.step(steps_prof, dt)
    torch.cuda.synchronize()
    prof = s.profile_read()
    s.profile(False)

    # ---- e2e through the public API: every step's state comes in from pinned host memory and its
    # result goes back to pinned host memory (Solver.advance_host_states: the copies of step k+1 and
    # k-1 overlap the kernels of step k)
    s.close()
    s = wl.solver(head)
    host_in = s.state64().cpu().pin_memory()
    host_out = [torch.empty_like(host_in).pin_memory() for _ in range(2)]
    e2e_steps = max(2, min(K, 10))
    s.advance_host_states([host_in] * 2, host_out, dt)  # warm-up: staging buffers, streams
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.advance_host_states([host_in] * e2e_steps, [host_out[k % 2] for k in range(e2e_steps)], dt)
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = aggregate_rate(cells, e2e_steps, t_e2e, world)
    bytes_io = host_in.numel() * 8
    s.close()
    del s

    # ---- the other precision on the same workload; error of the mixed run against the FP64 run
    K2 = max(1, min(K, args.fp64_steps if other == "fp64" else K))
    s2 = wl.solver(other)
    s2.step(min(W, 1), dt)
    t2 = time_steps(s2, K2, dt, torch)
    s2.close()
    s2 = wl.solver(other)
    s2.step(W + K, dt)
    q_other = s2.state64()
    s2.close()
    del s2
    q_mixed, q64 = (q_head, q_other) if head == "mixed" else (q_other, q_head)
    diff = q_mixed - q64
    nv = q64.shape[0]
    l2 = [float(torch.linalg.vector_norm(diff[v]) / torch.linalg.vector_norm(q64[v])) for v in range(nv)]
    linf = [float(diff[v].abs().max() / q64[v].abs().max()) for v in range(nv)]
    long_err = None
    if args.error_steps:
        # the configuration's own run length: both precisions from the initial state
        runs = {}
        for prec in ("mixed", "fp64"):
            s3 = wl.solver(prec)
            s3.step(args.error_steps, dt)
            runs[prec] = s3.state64()
            s3.close()
        d3 = runs["mixed"] - runs["fp64"]
        long_err = {"steps": args.error_steps,
                    "l2": [float(torch.linalg.vector_norm(d3[v]) / torch.linalg.vector_norm(runs["fp64"][v]))
                           for v in range(nv)],
                    "linf": [float(d3[v].abs().max() / runs["fp64"][v].abs().max()) for v in range(nv)],
                    "finite": bool(torch.isfinite(runs["mixed"]).all() and torch.isfinite(runs["fp64"]).all())}
        del runs, d3

    # ---- roofline: the whole RK3 step and the dominant kernel family
    peak, peak_kind = load_peaks()
    t_step = t / K
    bstage = wl.alg_bytes[head]
    achieved_step = cells * 3 * bstage / t_step / 1e9
    if wl.plan.ndim == 3:
        e = 4 if head == "mixed" else 8
        fam_bytes = {"weno_x": 5 * e * 2, "weno_y": 5 * e * 3, "weno_z": 5 * e * 3,
                     "central_rk": 5 * (e + e + 8 + 8 + e) if wl.plan.conv == "weno5js" else 5 * (e + 8 + 8 + e),
                     "halo": 0}
    else:
        e = 4 if head == "mixed" else 8
        fam_bytes = {"central_rk": 4 * (e + 8 + 8 + 8 + 8) + 8 * 2, "halo": 0}
    dom = max((f for f in prof if fam_bytes.get(f, 0) > 0), key=lambda f: prof[f][0], default=None)
    roof = None
    if dom:
        ms, cnt = prof[dom]
        per_launch = ms / cnt / 1e3
        ach = cells * fam_bytes[dom] / per_launch / 1e9
        traffic, tsrc = None, None
        if wl.name == "tgv_weno256" and head == "mixed" and dom in DRAM_BYTES_PER_CELL_WENO_MIXED:
            traffic = DRAM_BYTES_PER_CELL_WENO_MIXED[dom] * cells / 1e9
            tsrc = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the same kernel at 192^3, per cell, "
                    "times this launch's cells")
        issue = None
        if wl.name == "tgv_weno256" and head == "mixed" and dom in THREAD_INST_PER_CELL_WENO_MIXED:
            # the instruction-issue roofline of the same kernel: one warp-instruction per scheduler per
            # clock at the median SM clock sampled during the timed region
            mhz = clk.summary().get("sm_mhz") or 2070.0
            inst = THREAD_INST_PER_CELL_WENO_MIXED[dom] * cells
            ach_i = inst / per_launch / 1e12
            peak_i = SM_COUNT * SCHEDULERS_PER_SM * WARP * mhz * 1e6 / 1e12
            issue = {"achieved": ach_i, "peak": peak_i, "unit": "T thread-instructions/s", "frac": ach_i / peak_i,
                     "thread_inst_per_cell": THREAD_INST_PER_CELL_WENO_MIXED[dom], "sm_mhz": mhz,
                     "source": "ncu smsp__inst_executed of the same kernel at 192^3, per cell"}
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "issue": issue,
                "peak_kind": peak_kind, "traffic": traffic, "traffic_unit": "GB per launch",
                "traffic_source": tsrc, "alg_bytes_per_cell": fam_bytes[dom],
                "avg_launch_ms": per_launch * 1e3,
                "step": {"achieved": achieved_step, "frac": achieved_step / peak,
                         "alg_bytes_per_cell_per_stage": bstage},
                "families_ms_per_step": {f: prof[f][0] / steps_prof for f in prof}}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            r = reference_cpu(wl, args.ref_steps, 0)
            cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"]}
        except Exception as ex:
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "unavailable", "sample": str(ex)[:200]}

    if rank == 0:
        vars_ = ["rho", "rhou0", "rhou1", "rhou2", "rhoE"] if nv == 5 else ["rho", "rhou0", "rhou1", "rhoE"]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": 1e3 * t / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (RK accumulator f64)" if head == "mixed" else "f64",
                "data": "synthetic: the problem's analytic initial condition",
                "config": dict(wl.config, parallelism="replicas" if world > 1 else "single"),
                "roofline": roof, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_io,
                        "d2h_bytes_per_step": bytes_io, "steps": e2e_steps,
                        "path": "Solver.advance_host_states: per step, cudaMemcpyAsync of the pinned host state to the "
                                "device, osb_set_state64 + osb_step(1) + osb_get_state64, cudaMemcpyAsync of the result "
                                "to pinned host memory; copies on their own streams overlap the previous/next step"},
                "gpu_launches": launches, "clocks": clk.summary(),
                other: {"value": world * cells * K2 / t2, "ms_per_step": 1e3 * t2 / K2, "steps": K2},
                "mixed_vs_fp64_speedup": ((value / world) / (cells * K2 / t2)) if head == "mixed" else
                ((cells * K2 / t2) / (value / world)),
                "error_vs_fp64": {"steps": W + K, "l2": l2, "linf": linf, "vars": vars_}}
        if long_err:
            line["error_vs_fp64_long"] = long_err
        print(json.dumps(line), flush=True)


def adjoint_arm(args, world, rank, local):
    """Gradient of the volume-integrated kinetic energy at T = 2 with respect to the initial velocity
    field, 3D Taylor-Green 128^3, Re = 1600, Mach 0.1, central scheme, FP64, checkpoints every 20
    steps.  dt = 2.5e-3 (800 steps): the stated 400 steps of 5e-3 exceed the acoustic stability
    limit of the scheme at 128^3 (|lambda|_max dt ~ 2.7 > sqrt(3)).  Reports gradient throughput
    (cell-steps per second of forward + checkpointed adjoint) and directional derivatives against
    central finite differences (h = 1e-6) along seeded random directions."""
    import torch
    from opensbli_gb300.adjoint import Rollout, kinetic_energy, state_from_velocity, tgv_base
    from opensbli_gb300.plan import tgv_plan
    from opensbli_gb300.runtime import Solver

    torch.cuda.set_device(local)
    n = args.n or 128
    T_end, every = 2.0, 20
    nsteps = args.adj_steps or 800
    dt = T_end / nsteps
    plan = tgv_plan(n, conv="central_skew", precision="fp64", Minf=0.1, Re=1600.0)
    s = Solver(plan)
    p, rho, base = tgv_base(plan, s.device)
    cells = plan.cells

    def J_of(vel):
        s.set_state64(state_from_velocity(vel, p, rho, plan.gama))
        s.step(nsteps, dt)
        return float(kinetic_energy(s.state64(), plan.delta))

    J_of(base)  # warm-up (graph capture, scratch allocation)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J0 = J_of(base)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0

    def grad():
        v = base.clone().requires_grad_(True)
        qT = Rollout.apply(state_from_velocity(v, p, rho, plan.gama), s, nsteps, dt, every)
        J = kinetic_energy(qT, plan.delta)
        J.backward()
        return float(J.detach()), v.grad.detach()

    grad()  # warm-up of the adjoint scratch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, g = grad()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    fd = []
    for seed in range(args.fd_dirs):
        d = torch.randn(base.shape, generator=torch.Generator(device=s.device).manual_seed(seed), device=s.device,
                        dtype=torch.float64)
        h = 1e-6
        f = (J_of(base + h * d) - J_of(base - h * d)) / (2 * h)
        a = float((g * d).sum())
        fd.append({"seed": seed, "fd": f, "adjoint": a, "rel_err": abs(f - a) / abs(a)})
    s.close()
    if rank == 0:
        line = {"metric": "gradient cell-steps/s (forward + checkpointed adjoint)", "value": cells * nsteps / t_grad,
                "unit": "cell-steps/s", "n_gpus": world, "steps": nsteps, "warmup": 1,
                "ms_per_step": 1e3 * t_grad / nsteps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic: the problem's analytic initial condition",
                "config": {"workload": "adjoint of 3D Taylor-Green %d^3, Re=1600, Mach 0.1, central 4th-order, RK3, "
                                       "J = volume-integrated kinetic energy at T=2, gradient w.r.t. the initial "
                                       "velocity field, checkpoints every %d steps" % (n, every),
                           "grid": [n, n, n], "dt": dt, "nsteps": nsteps, "T": T_end,
                           "dt_note": "400 steps of 5e-3 exceed the scheme's acoustic stability limit at 128^3"},
                "J": J, "J_forward_only": J0, "forward_ms_per_step": 1e3 * t_fwd / nsteps,
                "gradient_over_forward": t_grad / t_fwd,
                "fd_check": {"h": 1e-6, "directions": len(fd),
                             "max_rel_err": max((r["rel_err"] for r in fd), default=None), "dirs": fd}}
        print(json.dumps(line), flush=True)


def ensemble_arm(args, world, rank, local):
    """96 perturbed Taylor-Green instances, n drawn from {32,48,64,96}^3, central or WENO5-JS per
    instance (seeded), per-instance CFL-0.5 time steps, stepped by the batched kernels (one graph per
    step); against looping the single-plan solver over the same instances."""
    import torch
    from opensbli_gb300.batch import Ensemble, tgv_ensemble
    from opensbli_gb300.runtime import Solver

    torch.cuda.set_device(local)
    K, W = args.steps, args.warmup
    prec = args.precision or "mixed"
    plans, states, dts = tgv_ensemble(count=96, precision=prec, seed=0)
    cells = sum(p.cells for p in plans)
    ens = Ensemble(plans)
    for i, q in enumerate(states):
        ens.set_state64(i, q)
    ens.set_dt(dts)
    tuned = ens.autotune(reps=3)
    ens.step(W)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        a.record(ens.stream)
        ens.step(K)
        b.record(ens.stream)
        torch.cuda.synchronize()
    t = max_over_ranks(a.elapsed_time(b) / 1e3, world)
    launches = ens.launch_count()
    finite = all(bool(torch.isfinite(ens.state64(i)).all()) for i in range(len(plans)))
    # e2e through the public API: every state in from pinned host memory, one step, every state out
    host_in = [q.cpu().pin_memory() for q in states]
    host_out = [torch.empty_like(h).pin_memory() for h in host_in]
    torch.cuda.synchronize()
    e2e_steps = max(1, min(K, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for i, h in enumerate(host_in):
            ens.set_state64(i, h.to(ens.device, non_blocking=True))
        ens.step(1)
        for i, h in enumerate(host_out):
            h.copy_(ens.state64(i), non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    bytes_io = sum(h.numel() * 8 for h in host_in)
    ens.close()
    # looping the single-plan solver (autotuned per instance) over the same instances
    t_loop = 0.0
    for i, p in enumerate(plans):
        s = Solver(p)
        s.set_state64(states[i])
        s.autotune(reps=2)
        s.step(1, dts[i])
        torch.cuda.synchronize()
        a.record(s.stream)
        s.step(K, dts[i])
        b.record(s.stream)
        torch.cuda.synchronize()
        t_loop += a.elapsed_time(b) / 1e3
        s.close()
    if rank == 0:
        value = aggregate_rate(cells, K, t, world)
        sizes = {}
        for p in plans:
            key = "%d^3 %s" % (p.n[0], "weno" if p.conv == "weno5js" else "central")
            sizes[key] = sizes.get(key, 0) + 1
        line = {"metric": "aggregate cell-updates/s per RK3 step", "value": value, "unit": "cell-updates/s",
                "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": 1e3 * t / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (RK accumulator f64)" if prec == "mixed" else "f64",
                "data": "synthetic: Taylor-Green fields + seeded band-limited perturbations",
                "config": {"workload": "batched ensemble: 96 Taylor-Green instances, n in {32,48,64,96}^3 and scheme "
                                       "(central / WENO5-JS) drawn with seed 0, Gaussian velocity perturbation RMS "
                                       "1e-2 with |k| <= 4 (seed = instance), Minf=0.1, Re=1600, dt from CFL 0.5 per "
                                       "instance", "instances": sizes, "cells": cells, "precision": prec,
                           "l2": "inputs larger than L2 (%.0f MB of state)" % (cells * 5 * (4 if prec == "mixed" else 8) / 1e6)},
                "tuned_shapes": tuned, "gpu_launches": launches, "clocks": clk.summary(), "finite": finite,
                "loop_single_solver": {"value": world * cells * K / t_loop, "ms_per_step": 1e3 * t_loop / K},
                "batch_over_loop": t_loop / t,
                "e2e": {"value": world * cells * e2e_steps / t_e2e, "unit": "cell-updates/s",
                        "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io, "steps": e2e_steps,
                        "path": "Ensemble.set_state64 (pinned host -> device) x96 + Ensemble.step(1) + state64 -> "
                                "pinned host x96"}}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--config", default="tgv_weno256",
                    choices=["tgv_weno256", "tgv_central64", "katzer512", "katzer512_adaptive", "tgv_adjoint128",
                             "tgv_batch96", "channel129", "shock_reflection"])
    ap.add_argument("--precision", default=None, choices=["mixed", "fp64"], help="tgv_batch96: precision")
    ap.add_argument("--adj-steps", type=int, default=None, help="tgv_adjoint128: RK3 steps to T=2 (default 800)")
    ap.add_argument("--fd-dirs", type=int, default=16, help="tgv_adjoint128: finite-difference directions")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--ref-steps", type=int, default=None,
                    help="timed steps of the host-core reference sample (default: 2 at 256^3, 40 otherwise)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--error-steps", type=int, default=None,
                    help="also run both precisions this many steps from the initial state and report the error "
                         "(default: the configuration's run length, 1000 steps, for tgv_weno256 at N=1; 0 elsewhere)")
    args = ap.parse_args()
    if args.ref_steps is None:
        args.ref_steps = 2 if args.config == "tgv_weno256" else 40
    world, rank, local = dist_init()
    if args.error_steps is None:
        # the accuracy bar is stated after the full run length; replicas (N > 1) repeat the N=1 numbers
        args.error_steps = 1000 if (args.config == "tgv_weno256" and world == 1 and args.n in (None, 256)) else 0
    if args.config == "tgv_batch96":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference runs one block per process; "
                                  "its ensemble throughput is the single-block figure of the other configs"}))
        else:
            ensemble_arm(args, world, rank, local)
    elif args.config == "tgv_adjoint128":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint of its time loop"}))
        else:
            adjoint_arm(args, world, rank, local)
    elif args.impl == "reference":
        ref_arm(args, world, rank)
    else:
        own_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
