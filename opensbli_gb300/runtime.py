"""ctypes binding of libosbli_gb300 (include/osb_gb300.h) and a torch-owned solver state.

`Solver(plan)` allocates the conserved-variable arrays as torch tensors on the current CUDA device
in the layout the library reports, binds them, and exposes the time loop (`step`), reductions,
residual evaluation and FP64 state access.  There is no CPU fallback: constructing a Solver
without a CUDA device or without the built library raises.
"""
import ctypes
import os

import torch

from . import build as _build

OSB_ABI_VERSION = 8
ERRORS = {
    -1: "invalid plan or argument",
    -2: "unsupported kernel pattern",
    -3: "CUDA error",
    -4: "field not bound",
    -5: "device wait timed out",
    -6: "non-finite value in the state",
    -7: "problem larger than a fixed-size scratch array",
}

CONV = {"central_skew": 0, "weno5js": 1, "teno5": 2, "weno5z": 3, "teno6": 4}
VISC = {"none": 0, "const": 1, "sutherland": 2, "power": 3}
AVG = {"roe": 0, "simple": 1}
RK = {"rk3": 0, "ls_rk3": 1}
BC = {"periodic": 0, "symmetry": 1, "inlet_pressure_extrapolate": 2, "extrapolation": 3, "isothermal_wall": 4,
      "dirichlet": 5, "adiabatic_wall": 6}
PREC = {"fp64": 0, "mixed": 1}
CLOSURE = {"reduced_access": 0, "carpenter": 1, "none": 2}
FILTER = {"none": 0, "weno5_constant": 1}
RED = {"ke": 0, "enstrophy": 1, "nancheck": 2}


class PlanDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int),
        ("ndim", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("delta", ctypes.c_double * 3),
        ("conv", ctypes.c_int),
        ("visc", ctypes.c_int),
        ("rk", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("bc", (ctypes.c_int * 2) * 3),
        ("gama", ctypes.c_double),
        ("Minf", ctypes.c_double),
        ("Re", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("weno_eps", ctypes.c_double),
        ("teno_ct", ctypes.c_double),
        ("teno_eps", ctypes.c_double),
        ("rk_a", ctypes.c_double * 3),
        ("rk_b", ctypes.c_double * 3),
        ("use_graphs", ctypes.c_int),
        ("Twall", ctypes.c_double),
        ("SuthT", ctypes.c_double),
        ("RefT", ctypes.c_double),
        ("dirichlet_state", (ctypes.c_double * 5) * 2),
        ("dirichlet_x_switch", ctypes.c_double),
        ("teno_adaptive", ctypes.c_int),
        ("teno_a1", ctypes.c_double),
        ("teno_a2", ctypes.c_double),
        ("sensor_eps", ctypes.c_double),
        ("shock_fp64", ctypes.c_double),
        ("dirichlet_ke", ctypes.c_int),
        ("body_force", ctypes.c_double * 5),
        ("closure", (ctypes.c_int * 2) * 3),
        ("filter", ctypes.c_int),
        ("filter_control", ctypes.c_double),
        ("visc_exp", ctypes.c_double),
        ("forcing", ctypes.c_double * 3),
        ("averaging", ctypes.c_int),
        ("cartesian", ctypes.c_int),
        ("dirichlet_x0", (ctypes.c_double * 5) * 2),
    ]


class Layout(ctypes.Structure):
    _fields_ = [
        ("numel", ctypes.c_int64),
        ("offset", ctypes.c_int64),
        ("stride_y", ctypes.c_int64),
        ("stride_z", ctypes.c_int64),
        ("halo", ctypes.c_int * 3),
        ("nvar", ctypes.c_int),
        ("state_bytes", ctypes.c_int),
    ]


EXPORTS = (
    "osb_query_layout", "osb_create", "osb_bind_field", "osb_set_stream", "osb_init_tgv", "osb_set_state64",
    "osb_set_state64_padded", "osb_set_coordinate",
    "osb_get_state64", "osb_teno_cutoff", "osb_step", "osb_residual", "osb_reduce", "osb_launch_count", "osb_profile", "osb_profile_read",
    "osb_set_weno_shape", "osb_get_weno_shape", "osb_set_central_shape", "osb_get_central_shape", "osb_autotune",
    "osb_adjoint_residual", "osb_adjoint_step", "osb_probe", "osb_set_tma", "osb_tma_active", "osb_get_error",
    "osb_destroy",
    "osb_batch_create", "osb_batch_set_stream", "osb_batch_set_dt", "osb_batch_set_state64", "osb_batch_get_state64",
    "osb_batch_step", "osb_batch_autotune", "osb_batch_get_shape", "osb_batch_launch_count", "osb_batch_get_error",
    "osb_batch_destroy",
)
# launch shapes of the WENO flux kernels (osb_set_weno_shape)
WENO_SHAPES = {"tile": 0, "march4": 1, "march8": 2}
PROFILE_FAMILIES = ["halo", "weno_x", "weno_y", "weno_z", "central_rk", "other"]

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the shared library (building it first if asked and needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libosbli_gb300.so is not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.osb_query_layout.argtypes = [ctypes.POINTER(PlanDesc), ctypes.POINTER(Layout)]
    lib.osb_create.argtypes = [ctypes.POINTER(PlanDesc), ctypes.POINTER(vp)]
    lib.osb_bind_field.argtypes = [vp, ip, vp]
    lib.osb_set_stream.argtypes = [vp, vp]
    lib.osb_init_tgv.argtypes = [vp]
    lib.osb_set_state64.argtypes = [vp, ip, vp]
    lib.osb_set_state64_padded.argtypes = [vp, ip, vp, ip]
    lib.osb_set_coordinate.argtypes = [vp, ip, vp, ip]
    lib.osb_get_state64.argtypes = [vp, ip, vp]
    lib.osb_teno_cutoff.argtypes = [vp, vp]
    lib.osb_step.argtypes = [vp, ip, dp]
    lib.osb_residual.argtypes = [vp, vp]
    lib.osb_reduce.argtypes = [vp, ip, ctypes.POINTER(dp)]
    lib.osb_launch_count.argtypes = [vp]
    lib.osb_launch_count.restype = ctypes.c_int64
    lib.osb_profile.argtypes = [vp, ip]
    lib.osb_profile_read.argtypes = [vp, ctypes.POINTER(dp), ctypes.POINTER(ctypes.c_int64), ip]
    lib.osb_set_weno_shape.argtypes = [vp, ip, ip, ip]
    lib.osb_get_weno_shape.argtypes = [vp, ip, ctypes.POINTER(ip), ctypes.POINTER(ip)]
    lib.osb_set_central_shape.argtypes = [vp, ip]
    lib.osb_get_central_shape.argtypes = [vp, ctypes.POINTER(ip)]
    lib.osb_autotune.argtypes = [vp, ip, ctypes.POINTER(dp)]
    lib.osb_adjoint_residual.argtypes = [vp, vp, vp]
    lib.osb_probe.argtypes = [vp, ip, ctypes.POINTER(ip), ctypes.POINTER(dp)]
    lib.osb_set_tma.argtypes = [vp, ip]
    lib.osb_tma_active.argtypes = [vp]
    lib.osb_adjoint_step.argtypes = [vp, dp, vp, vp]
    lib.osb_get_error.argtypes = [vp, ctypes.c_char_p, ip]
    lib.osb_batch_create.argtypes = [ctypes.POINTER(PlanDesc), ip, ctypes.POINTER(vp)]
    lib.osb_batch_set_stream.argtypes = [vp, vp]
    lib.osb_batch_set_dt.argtypes = [vp, ctypes.POINTER(dp)]
    lib.osb_batch_set_state64.argtypes = [vp, ip, vp]
    lib.osb_batch_get_state64.argtypes = [vp, ip, vp]
    lib.osb_batch_step.argtypes = [vp, ip]
    lib.osb_batch_autotune.argtypes = [vp, ip, ctypes.POINTER(dp)]
    lib.osb_batch_get_shape.argtypes = [vp, ctypes.POINTER(ip), ip]
    lib.osb_batch_launch_count.argtypes = [vp]
    lib.osb_batch_launch_count.restype = ctypes.c_int64
    lib.osb_batch_get_error.argtypes = [vp, ctypes.c_char_p, ip]
    lib.osb_batch_destroy.argtypes = [vp]
    lib.osb_batch_destroy.restype = None
    lib.osb_destroy.argtypes = [vp]
    lib.osb_destroy.restype = None
    for name in EXPORTS:
        if name not in ("osb_launch_count", "osb_destroy", "osb_batch_launch_count", "osb_batch_destroy"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


class OSBError(RuntimeError):
    pass


def make_plan_desc(plan):
    """Fill the C plan struct from a Plan (opensbli_gb300.plan.Plan)."""
    d = PlanDesc()
    d.abi_version = OSB_ABI_VERSION
    d.ndim = plan.ndim
    for i in range(3):
        d.n[i] = plan.n[i]
        d.delta[i] = plan.delta[i]
    d.conv = CONV[plan.conv]
    d.visc = VISC[plan.visc]
    d.rk = RK[plan.rk]
    d.precision = PREC[plan.precision]
    for a in range(3):
        for s in range(2):
            d.bc[a][s] = BC[plan.bc[a][s]]
    d.gama, d.Minf, d.Re, d.Pr = plan.gama, plan.Minf, plan.Re, plan.Pr
    d.weno_eps = plan.weno_eps
    d.teno_ct, d.teno_eps = plan.teno_ct, plan.teno_eps
    for s in range(3):
        d.rk_a[s] = plan.rk_a[s]
        d.rk_b[s] = plan.rk_b[s]
    d.use_graphs = 1 if plan.use_graphs else 0
    d.Twall, d.SuthT, d.RefT = plan.Twall, plan.SuthT, plan.RefT
    for v in range(len(plan.dirichlet_lo)):
        d.dirichlet_state[0][v] = plan.dirichlet_lo[v]
        d.dirichlet_state[1][v] = plan.dirichlet_hi[v]
    d.dirichlet_x_switch = plan.dirichlet_x_switch
    d.teno_adaptive = 1 if plan.teno_adaptive else 0
    d.teno_a1, d.teno_a2, d.sensor_eps = plan.teno_a1, plan.teno_a2, plan.sensor_eps
    d.shock_fp64 = plan.shock_fp64
    d.dirichlet_ke = 1 if plan.dirichlet_ke else 0
    for k, v in enumerate(plan.body_force or (0.0,) * 5):
        d.body_force[k] = v
    for a in range(len(plan.closure)):
        for side in range(2):
            d.closure[a][side] = CLOSURE[plan.closure[a][side]]
    d.filter = FILTER[plan.filter]
    d.filter_control = plan.filter_control
    d.visc_exp = plan.visc_exp
    for k, v in enumerate(plan.forcing or (0.0,) * 3):
        d.forcing[k] = v
    d.averaging = AVG[plan.averaging]
    d.cartesian = 1 if plan.x1_grid == "uniform" else 0
    for side, st in enumerate(plan.dirichlet_x0 or ()):
        for v, x in enumerate(st):
            d.dirichlet_x0[side][v] = x
    return d


class Solver:
    """One block's flow state on the current CUDA device, advanced by libosbli_gb300."""

    def __init__(self, plan, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("opensbli_gb300 needs a CUDA device; there is no CPU path")
        self.lib = load()
        self.plan = plan
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.desc = make_plan_desc(plan)
        lay = Layout()
        self._check(self.lib.osb_query_layout(ctypes.byref(self.desc), ctypes.byref(lay)), ctx=None)
        self.layout = lay
        self.dtype = torch.float32 if lay.state_bytes == 4 else torch.float64
        with torch.cuda.device(self.device):
            h = ctypes.c_void_p()
            self._check(self.lib.osb_create(ctypes.byref(self.desc), ctypes.byref(h)), ctx=None)
            self.ctx = h
            self.fields = [torch.zeros(lay.numel, dtype=self.dtype, device=self.device) for _ in range(lay.nvar)]
            for v, t in enumerate(self.fields):
                self._check(self.lib.osb_bind_field(self.ctx, v, ctypes.c_void_p(t.data_ptr())))
            # a dedicated stream: CUDA graphs cannot be captured on the legacy default stream
            self.stream = torch.cuda.Stream(self.device)
            self._check(self.lib.osb_set_stream(self.ctx, ctypes.c_void_p(self.stream.cuda_stream)))
            torch.cuda.synchronize(self.device)

    # -- helpers
    def _check(self, rc, ctx="self"):
        if rc == 0:
            return
        msg = ERRORS.get(rc, "error %d" % rc)
        c = self.ctx if ctx == "self" else None
        if c is not None:
            buf = ctypes.create_string_buffer(512)
            self.lib.osb_get_error(c, buf, 512)
            if buf.value:
                msg += ": " + buf.value.decode()
        if rc == -2:
            raise NotImplementedError(msg)
        raise OSBError(msg)

    @property
    def shape(self):
        if self.plan.ndim == 1:
            return (self.plan.n[0],)
        if self.plan.ndim == 2:
            return (self.plan.n[1], self.plan.n[0])
        return (self.plan.n[2], self.plan.n[1], self.plan.n[0])

    def interior(self, var):
        """View of the interior of bound variable `var` as [z][y][x] ([y][x] in 2D), state precision."""
        lay = self.layout
        if self.plan.ndim == 1:
            return torch.as_strided(self.fields[var], self.shape, (1,), lay.offset)
        if self.plan.ndim == 2:
            return torch.as_strided(self.fields[var], self.shape, (lay.stride_y, 1), lay.offset)
        n0, n1, n2 = self.plan.n
        return torch.as_strided(self.fields[var], (n2, n1, n0), (lay.stride_z, lay.stride_y, 1), lay.offset)

    # -- stream ordering: library work runs on self.stream; it waits for the caller's current stream
    # before each call, and the caller's stream waits for it afterwards.
    def _in(self):
        self.stream.wait_stream(torch.cuda.current_stream(self.device))

    def _out(self):
        torch.cuda.current_stream(self.device).wait_stream(self.stream)

    # -- API
    def init_tgv(self):
        self._in()
        self._check(self.lib.osb_init_tgv(self.ctx))
        self._out()

    @staticmethod
    def _check_shape(t, shape, what):
        # the kernels index the array from the plan's sizes: a smaller array would be read past its end
        if tuple(t.shape) != tuple(shape):
            raise ValueError("%s of shape %s, the block needs %s" % (what, tuple(t.shape), tuple(shape)))

    @staticmethod
    def _pinned64(t):
        return (isinstance(t, torch.Tensor) and t.device.type == "cpu" and t.dtype == torch.float64 and
                t.is_contiguous() and t.is_pinned())

    def set_state64(self, q):
        """q: FP64 tensor/array [nvar][z][y][x] (interior).  A page-locked (pinned) host tensor is read by
        the library's kernels over the host link without a staging copy; the call then waits for them,
        so the buffer may be reused on return."""
        pinned = self._pinned64(q)
        if not pinned:
            q = torch.as_tensor(q, dtype=torch.float64).to(self.device).contiguous()
        self._check_shape(q, (self.layout.nvar,) + self.shape, "state")
        self._in()
        for v in range(self.layout.nvar):
            self._check(self.lib.osb_set_state64(self.ctx, v, ctypes.c_void_p(q[v].data_ptr())))
        if pinned:
            self.stream.synchronize()
        else:
            q.record_stream(self.stream)
        self._out()

    def set_state64_padded(self, q, h):
        """q: FP64 [nvar][...] including a halo of width h on every side (the initialisation kernel's
        range)."""
        q = torch.as_tensor(q, dtype=torch.float64).to(self.device).contiguous()
        self._check_shape(q, (self.layout.nvar,) + tuple(k + 2 * int(h) for k in self.shape), "padded state")
        self._in()
        for v in range(self.layout.nvar):
            self._check(self.lib.osb_set_state64_padded(self.ctx, v, ctypes.c_void_p(q[v].data_ptr()), int(h)))
        q.record_stream(self.stream)
        self._out()

    def state_names(self):
        """OPS dat names of the conserved variables on block 0 (rho_B0, rhou0_B0, ...)."""
        nv = self.layout.nvar
        return ["rho_B0", "rhou0_B0", "rhou1_B0", "rhoE_B0"] if nv == 4 else \
            ["rho_B0", "rhou0_B0", "rhou1_B0", "rhou2_B0", "rhoE_B0"]

    def write_ops_hdf5(self, path, extra=None, halo=5, block_name="opensbliblock00"):
        """Write the FP64 state as an OPS block file (the layout of the generated code's
        ops_fetch_block_hdf5_file / ops_fetch_dat_hdf5_file calls): one dat per conserved variable, plus
        `extra` = {dat name: FP64 interior array} (coordinates, sensors).  Halos are `halo` deep on
        every side: periodic axes carry the periodic images, other axes zeros (the boundary kernels
        recompute halos on restart)."""
        import numpy as np
        from . import hdf5
        q = self.state64().cpu().numpy()
        arrays = {n: q[v] for v, n in enumerate(self.state_names())}
        for k, a in (extra or {}).items():
            arrays[k] = np.asarray(a, dtype=np.float64)
        nd = self.plan.ndim
        modes = [("wrap" if self.plan.bc[d][0] == "periodic" else "constant") for d in range(nd)][::-1]
        padded = []
        for a in arrays.values():
            if a.shape != self.shape:
                raise ValueError("extra dat of shape %s, the block is %s" % (a.shape, self.shape))
            for ax, m in enumerate(modes):
                w = [(0, 0)] * nd
                w[ax] = (halo, halo)
                a = np.pad(a, w, mode=m)
            padded.append(a)
        hdf5.write_ops_state(path, list(arrays), padded, tuple(self.plan.n[:nd]), halo, block_name)

    def read_ops_hdf5(self, path, block_name="opensbliblock00"):
        """Set the state from an OPS block file holding the conserved dats (as written by
        write_ops_hdf5 or by the generated code); the halos in the file are not used."""
        import numpy as np
        from . import hdf5
        arrays, halo, npts = hdf5.read_ops_state(path, self.state_names(), block_name)
        if tuple(npts) != tuple(self.plan.n[:self.plan.ndim]):
            raise ValueError("%s holds a %s block, the plan is %s" % (path, npts, self.plan.n[:self.plan.ndim]))
        sl = (slice(halo, -halo),) * self.plan.ndim if halo else (slice(None),) * self.plan.ndim
        self.set_state64(np.stack([a[sl] for a in arrays]))

    def set_coordinate(self, x1, h=4):
        """Blocks stretched in x1: the x1 coordinate, FP64 [n1+2h][n0+2h] on 2D blocks, the line
        [n1+2h] (x1 depends on j alone) on 3D wall-bounded blocks; evaluates the metrics."""
        x = torch.as_tensor(x1, dtype=torch.float64).to(self.device).contiguous()
        if self.plan.ndim == 3:
            self._check_shape(x, (self.plan.n[1] + 2 * int(h),), "coordinate line")
        else:
            self._check_shape(x, tuple(k + 2 * int(h) for k in self.shape), "coordinate")
        self._in()
        self._check(self.lib.osb_set_coordinate(self.ctx, 1, ctypes.c_void_p(x.data_ptr()), int(h)))
        x.record_stream(self.stream)
        self._out()

    def state64(self, out=None):
        """The FP64 state [nvar][z][y][x].  With `out` a page-locked (pinned) host tensor of that shape,
        the kernels write it directly over the host link and the call waits for them."""
        shape = (self.layout.nvar,) + self.shape
        pinned = out is not None
        if pinned and not (self._pinned64(out) and tuple(out.shape) == shape):
            raise ValueError("out must be a contiguous pinned FP64 host tensor of shape %s" % (shape,))
        self._in()
        if out is None:
            with torch.cuda.stream(self.stream):
                out = torch.empty(shape, dtype=torch.float64, device=self.device)
        for v in range(self.layout.nvar):
            self._check(self.lib.osb_get_state64(self.ctx, v, ctypes.c_void_p(out[v].data_ptr())))
        if pinned:
            self.stream.synchronize()
        self._out()
        return out

    def advance_host_states(self, inputs, outputs, dt, nsteps=1):
        """Advance independent states held in page-locked host memory: outputs[k] = the state after
        nsteps RK3 steps of size dt from inputs[k] (FP64 [nvar][z][y][x], contiguous pinned host
        tensors; an input tensor may be listed more than once).  The jobs are pipelined over three
        streams: while job k computes, the copy engines bring job k+1's state in and take job k-1's
        result out, so the host link's time hides behind the kernels instead of adding to them.  The
        solver's own state is left holding the last job's result.  Returns when every output has
        been written."""
        shape = (self.layout.nvar,) + self.shape
        for t in list(inputs) + list(outputs):
            if not (self._pinned64(t) and tuple(t.shape) == shape):
                raise ValueError("inputs and outputs must be contiguous pinned FP64 host tensors of shape %s" %
                                 (shape,))
        if len(inputs) != len(outputs):
            raise ValueError("one output per input")
        if not hasattr(self, "_pipe"):
            self._pipe = {
                "in": [torch.empty(shape, dtype=torch.float64, device=self.device) for _ in range(2)],
                "out": [torch.empty(shape, dtype=torch.float64, device=self.device) for _ in range(2)],
                "h2d": torch.cuda.Stream(self.device), "d2h": torch.cuda.Stream(self.device)}
        pp = self._pipe
        ev = lambda: torch.cuda.Event()  # noqa: E731
        loaded, consumed, computed, drained = [None, None], [None, None], [None, None], [None, None]
        self._in()
        pp["h2d"].wait_stream(self.stream)
        pp["d2h"].wait_stream(self.stream)
        for k, (src, dst) in enumerate(zip(inputs, outputs)):
            slot = k % 2
            with torch.cuda.stream(pp["h2d"]):
                if consumed[slot] is not None:
                    pp["h2d"].wait_event(consumed[slot])  # job k-2 has read this staging buffer
                pp["in"][slot].copy_(src, non_blocking=True)
                loaded[slot] = ev()
                loaded[slot].record(pp["h2d"])
            self.stream.wait_event(loaded[slot])
            for v in range(self.layout.nvar):
                self._check(self.lib.osb_set_state64(self.ctx, v, ctypes.c_void_p(pp["in"][slot][v].data_ptr())))
            consumed[slot] = ev()
            consumed[slot].record(self.stream)
            self._check(self.lib.osb_step(self.ctx, int(nsteps), float(dt)))
            if drained[slot] is not None:
                self.stream.wait_event(drained[slot])  # job k-2's result has left this buffer
            for v in range(self.layout.nvar):
                self._check(self.lib.osb_get_state64(self.ctx, v, ctypes.c_void_p(pp["out"][slot][v].data_ptr())))
            computed[slot] = ev()
            computed[slot].record(self.stream)
            with torch.cuda.stream(pp["d2h"]):
                pp["d2h"].wait_event(computed[slot])
                dst.copy_(pp["out"][slot], non_blocking=True)
                drained[slot] = ev()
                drained[slot].record(pp["d2h"])
        pp["d2h"].synchronize()
        pp["h2d"].synchronize()
        self.stream.synchronize()
        self._out()

    def teno_cutoff(self):
        """The adaptive TENO cut-off C_T of the current state, FP64 [n1][n0] (2D) or [n2][n1][n0] (3D)
        for plans with teno_adaptive (the reference's TENO_B0 output field)."""
        self._in()
        with torch.cuda.stream(self.stream):
            out = torch.empty(self.shape, dtype=torch.float64, device=self.device)
        self._check(self.lib.osb_teno_cutoff(self.ctx, ctypes.c_void_p(out.data_ptr())))
        self._out()
        return out

    def step(self, nsteps, dt):
        self._in()
        self._check(self.lib.osb_step(self.ctx, int(nsteps), float(dt)))
        self._out()

    def residual(self):
        self._in()
        with torch.cuda.stream(self.stream):
            out = torch.empty((self.layout.nvar,) + self.shape, dtype=self.dtype, device=self.device)
        self._check(self.lib.osb_residual(self.ctx, ctypes.c_void_p(out.data_ptr())))
        self._out()
        return out

    def reduce(self, what):
        v = ctypes.c_double()
        self._in()
        self._check(self.lib.osb_reduce(self.ctx, RED[what], ctypes.byref(v)))
        return v.value

    def profile(self, enable=True):
        self._check(self.lib.osb_profile(self.ctx, 1 if enable else 0))

    def profile_read(self):
        """{family: (total_ms, launches)} accumulated since profile(True)."""
        ms = (ctypes.c_double * 8)()
        cnt = (ctypes.c_int64 * 8)()
        n = self.lib.osb_profile_read(self.ctx, ms, cnt, 8)
        return {PROFILE_FAMILIES[f]: (ms[f], int(cnt[f])) for f in range(min(n, len(PROFILE_FAMILIES))) if cnt[f]}

    def launch_count(self):
        return int(self.lib.osb_launch_count(self.ctx))

    def probe(self, requests):
        """Point values from the FP64 state: requests = [(what, i, j, k), ...] with what a conserved
        variable index or one of opensbli_gb300.monitor.DERIVED's codes; returns a list of floats."""
        n = len(requests)
        if n == 0:
            return []
        flat = (ctypes.c_int * (4 * n))(*[int(x) for r in requests for x in r])
        out = (ctypes.c_double * n)()
        self._in()
        self._check(self.lib.osb_probe(self.ctx, n, flat, out))
        return list(out)

    def set_weno_shape(self, d, kind, seg=32):
        """Launch shape of the direction-d WENO flux kernel: kind in WENO_SHAPES, seg cells per line
        segment for the line-marching shapes."""
        self._check(self.lib.osb_set_weno_shape(self.ctx, int(d), WENO_SHAPES[kind], int(seg)))

    def weno_shape(self, d):
        k, sg = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.osb_get_weno_shape(self.ctx, int(d), ctypes.byref(k), ctypes.byref(sg)))
        return {v: n for n, v in WENO_SHAPES.items()}[k.value], sg.value

    def set_central_shape(self, ty):
        """Tile height (8 or 16) of the fused central/RK kernel."""
        self._check(self.lib.osb_set_central_shape(self.ctx, int(ty)))

    def set_tma(self, enable=True):
        """Select TMA plane loads (default) or register-staged loads in the fused central/RK kernel."""
        self._check(self.lib.osb_set_tma(self.ctx, 1 if enable else 0))

    def tma_active(self):
        return bool(self.lib.osb_tma_active(self.ctx))

    def central_shape(self):
        ty = ctypes.c_int()
        self._check(self.lib.osb_get_central_shape(self.ctx, ctypes.byref(ty)))
        return ty.value

    def autotune(self, reps=5):
        """Time the candidate launch shapes on the bound state and keep the fastest; returns
        {"weno_x"|"weno_y"|"weno_z": (kind, seg, ms per launch), "central": (ty, ms per launch)}
        for the kernels the plan uses (empty for 2D plans)."""
        best = (ctypes.c_double * 4)()
        self._in()
        self._check(self.lib.osb_autotune(self.ctx, int(reps), best))
        self._out()
        if self.plan.ndim != 3:
            return {}
        out = {"central": (self.central_shape(), best[3])}
        if self.plan.conv in ("weno5js", "weno5z"):
            for d, name in enumerate(("weno_x", "weno_y", "weno_z")):
                out[name] = self.weno_shape(d) + (best[d],)
        return out

    # -- discrete adjoint (FP64 periodic central plans)
    def _dense64(self, a):
        shape = (self.layout.nvar,) + self.shape
        t = torch.as_tensor(a, dtype=torch.float64).to(self.device).reshape(shape).contiguous()
        return t

    def adjoint_residual(self, lam):
        """(dR/dq)^T lam at the bound state; lam FP64 [5][z][y][x]."""
        lam = self._dense64(lam)
        self._in()
        with torch.cuda.stream(self.stream):
            out = torch.empty_like(lam)
        self._check(self.lib.osb_adjoint_residual(self.ctx, ctypes.c_void_p(lam.data_ptr()),
                                                  ctypes.c_void_p(out.data_ptr())))
        lam.record_stream(self.stream)
        self._out()
        return out

    def adjoint_step(self, lam, dt):
        """(dPhi/dq)^T lam for one RK3 step Phi of size dt from the bound state (left unchanged)."""
        lam = self._dense64(lam)
        self._in()
        with torch.cuda.stream(self.stream):
            out = torch.empty_like(lam)
        self._check(self.lib.osb_adjoint_step(self.ctx, float(dt), ctypes.c_void_p(lam.data_ptr()),
                                              ctypes.c_void_p(out.data_ptr())))
        lam.record_stream(self.stream)
        self._out()
        return out

    def close(self):
        if getattr(self, "ctx", None):
            torch.cuda.synchronize(self.device)
            self.lib.osb_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
