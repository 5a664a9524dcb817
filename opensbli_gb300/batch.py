"""Ensemble: many independent periodic 3D blocks stepped together by the batched kernels
(osb_batch_* in the C ABI: per RK3 stage one launch per halo axis and persistent tile-queue launches
for the WENO directions and the fused central/RK update over all instances; one CUDA graph per
step).

    ens = Ensemble([tgv_plan(32), tgv_plan(96, conv="weno5js"), ...])
    ens.set_state64(i, q_i)          # FP64 [5][n][n][n] per instance
    ens.set_dt([dt_0, dt_1, ...])
    ens.autotune()
    ens.step(500)
    q = ens.state64(i)

Instances may differ in size, scheme (central skew-symmetric or WENO5-JS) and constants; they share
the precision and the RK3 coefficients.  tgv_ensemble() builds the perturbed Taylor-Green ensemble
of the reference's TGV script with seeded sizes, schemes and velocity perturbations.
"""
import ctypes
import math

import torch

from . import runtime
from .plan import tgv_plan


class Ensemble:
    def __init__(self, plans, device=None):
        self.lib = runtime.load()
        self.plans = list(plans)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float32 if self.plans[0].precision == "mixed" else torch.float64
        descs = (runtime.PlanDesc * len(self.plans))()
        for i, p in enumerate(self.plans):
            descs[i] = runtime.make_plan_desc(p)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            self._check(self.lib.osb_batch_create(descs, len(self.plans), ctypes.byref(h)), None)
            self.b = h
            self.stream = torch.cuda.Stream(self.device)
            self._check(self.lib.osb_batch_set_stream(self.b, ctypes.c_void_p(self.stream.cuda_stream)))
            torch.cuda.synchronize(self.device)

    def _check(self, rc, b="self"):
        if rc == 0:
            return
        msg = runtime.ERRORS.get(rc, "error %d" % rc)
        h = self.b if b == "self" else None
        if h is not None:
            buf = ctypes.create_string_buffer(512)
            self.lib.osb_batch_get_error(h, buf, 512)
            if buf.value:
                msg += ": " + buf.value.decode()
        if rc == -2:
            raise NotImplementedError(msg)
        raise runtime.OSBError(msg)

    def __len__(self):
        return len(self.plans)

    @property
    def cells(self):
        return sum(p.cells for p in self.plans)

    def _in(self):
        self.stream.wait_stream(torch.cuda.current_stream(self.device))

    def _out(self):
        torch.cuda.current_stream(self.device).wait_stream(self.stream)

    def shape(self, i):
        n0, n1, n2 = self.plans[i].n
        return (5, n2, n1, n0)

    def set_state64(self, i, q):
        q = torch.as_tensor(q, dtype=torch.float64).to(self.device).reshape(self.shape(i)).contiguous()
        self._in()
        self._check(self.lib.osb_batch_set_state64(self.b, int(i), ctypes.c_void_p(q.data_ptr())))
        q.record_stream(self.stream)
        self._out()

    def state64(self, i):
        self._in()
        with torch.cuda.stream(self.stream):
            out = torch.empty(self.shape(i), dtype=torch.float64, device=self.device)
        self._check(self.lib.osb_batch_get_state64(self.b, int(i), ctypes.c_void_p(out.data_ptr())))
        self._out()
        return out

    def set_dt(self, dts):
        arr = (ctypes.c_double * len(self.plans))(*[float(x) for x in dts])
        self._in()
        self._check(self.lib.osb_batch_set_dt(self.b, arr))
        self.stream.synchronize()  # the host array is read by a stream-ordered copy

    def step(self, nsteps):
        self._in()
        self._check(self.lib.osb_batch_step(self.b, int(nsteps)))
        self._out()

    def autotune(self, reps=3):
        """Pick the batched kernels' tile shapes by timing them on the current states; returns
        {"weno_x"|"weno_y"|"weno_z": (kind, seg, ms), "central": (ty, zplanes, ms)}."""
        best = (ctypes.c_double * 4)()
        self._in()
        self._check(self.lib.osb_batch_autotune(self.b, int(reps), best))
        self._out()
        sh = self.shape_config()
        kinds = {v: k for k, v in runtime.WENO_SHAPES.items()}
        out = {"central": (sh[6], sh[7], best[3])}
        if any(p.conv == "weno5js" for p in self.plans):
            for d, name in enumerate(("weno_x", "weno_y", "weno_z")):
                out[name] = (kinds[sh[2 * d]], sh[2 * d + 1], best[d])
        return out

    def shape_config(self):
        out = (ctypes.c_int * 8)()
        self._check(self.lib.osb_batch_get_shape(self.b, out, 8))
        return list(out)

    def launch_count(self):
        return int(self.lib.osb_batch_launch_count(self.b))

    def close(self):
        if getattr(self, "b", None):
            torch.cuda.synchronize(self.device)
            self.lib.osb_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def band_limited_field(n, kmax, seed, device, amplitude):
    """A Gaussian random field on the periodic n^3 grid with Fourier modes |k| <= kmax only, scaled to
    the given RMS amplitude ([3][n][n][n], one field per velocity component)."""
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    out = []
    k = torch.fft.fftfreq(n, d=1.0 / n)
    KZ, KY, KX = torch.meshgrid(k, k, k, indexing="ij")
    mask = (KX ** 2 + KY ** 2 + KZ ** 2) <= kmax * kmax
    for _ in range(3):
        w = torch.randn((n, n, n), generator=g, dtype=torch.float64)
        f = torch.fft.ifftn(torch.fft.fftn(w) * mask).real
        f = f * (amplitude / f.pow(2).mean().sqrt())
        out.append(f)
    return torch.stack(out).to(device)


def tgv_ensemble(count=96, sizes=(32, 48, 64, 96), precision="mixed", seed=0, Minf=0.1, amplitude=1e-2, kmax=4,
                 cfl=0.5, device=None):
    """The perturbed Taylor-Green ensemble: instance i has n^3 points with n drawn uniformly from
    `sizes` and the scheme (central skew-symmetric or WENO5-JS) drawn by torch.Generator seeded with
    `seed`; its velocity is the Taylor-Green field plus a band-limited (|k| <= kmax) Gaussian
    perturbation of RMS `amplitude` seeded with i; dt from CFL `cfl` on the initial state.
    Returns (plans, initial states, dts)."""
    from .adjoint import state_from_velocity, tgv_base
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device="cpu").manual_seed(seed)
    ns = [sizes[int(j)] for j in torch.randint(len(sizes), (count,), generator=g)]
    schemes = ["central_skew" if int(j) == 0 else "weno5js" for j in torch.randint(2, (count,), generator=g)]
    plans, states, dts = [], [], []
    for i, (n, conv) in enumerate(zip(ns, schemes)):
        plan = tgv_plan(n, conv=conv, precision=precision, Minf=Minf)
        p, rho, vel = tgv_base(plan, dev)
        vel = vel + band_limited_field(n, kmax, i, dev, amplitude)
        q = state_from_velocity(vel, p, rho, plan.gama)
        a = torch.sqrt(plan.gama * p / rho)
        smax = float((vel.pow(2).sum(0).sqrt() + a).max())
        plans.append(plan)
        states.append(q)
        dts.append(cfl * min(plan.delta) / smax)
    return plans, states, dts
