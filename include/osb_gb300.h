/* osb_gb300.h -- C ABI of the GB300 backend for OpenSBLI's per-timestep hot path.
 *
 * The library replaces what the reference's OPSC writer (code_generation/opsc.py:250-282) emits
 * and what OPS runs for it: the per-stage kernel list of the generated solver
 * (code_generation/algorithm/algorithm.py:384-477) -- constituent relations, spatial residual,
 * Runge-Kutta update and boundary halos -- as hand-written sm_103a CUDA kernels.  A problem script
 * builds its TraditionalAlgorithmRK as before; opensbli_gb300.GB300Writer(alg) lowers it to an
 * osb_plan_desc and drives this ABI through ctypes.  Plain C types only; device pointers are
 * owned by the caller (torch tensors in the Python host) unless stated.
 *
 * Return codes: 0 ok, < 0 error (see OSB_E*); osb_get_error gives the message of the last error.
 * Threading: one context per CUDA stream, not thread-safe on the same context.
 */
#ifndef OSB_GB300_H
#define OSB_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define OSB_ABI_VERSION 8

/* error codes */
#define OSB_OK 0
#define OSB_EINVAL (-1)      /* bad plan or argument */
#define OSB_EUNSUPPORTED (-2) /* plan asks for a kernel pattern this backend does not implement */
#define OSB_ECUDA (-3)       /* CUDA runtime error */
#define OSB_ENOTBOUND (-4)   /* a field is missing */
#define OSB_ETIMEOUT (-5)    /* a bounded device wait gave up (device status word) */
#define OSB_ENONFINITE (-6)  /* NaN/Inf found by osb_reduce(OSB_RED_NANCHECK) */
#define OSB_ETOOLARGE (-7)   /* problem larger than a fixed-size scratch array (osb_reduce_noalloc) */

/* convective schemes: Central(4) skew-symmetric (schemes/spatial/scheme.py:187-271, core/parsing.py:75-111),
 * LLFWeno(5,'JS') (schemes/spatial/weno.py:474-521), LLFTeno(5) (schemes/spatial/teno.py:489-530) */
#define OSB_CONV_CENTRAL_SKEW 0
#define OSB_CONV_WENO5JS 1
#define OSB_CONV_TENO5 2
#define OSB_CONV_WENO5Z 3   /* WENO5-Z weights (weno.py:283-331), 3D blocks */
#define OSB_CONV_TENO6 4    /* LLFTeno(6), fixed cut-off (teno.py:94-192, 216-234), 3D blocks */
/* viscous terms: none, constant viscosity (taylor_green_vortex.py:18-19), Sutherland (katzer_SBLI.py:25),
 * the power law mu = T^visc_exp (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py:30) */
#define OSB_VISC_NONE 0
#define OSB_VISC_CONST 1
#define OSB_VISC_SUTHERLAND 2
#define OSB_VISC_POWER 3
/* time integration: RungeKutta(3) 2-register (schemes/temporal/rk_sbli.py:51-61, 117-124),
 * RungeKuttaLS(3,'SSP') (schemes/temporal/rk_LS.py:71-101, 155-166) */
#define OSB_RK3_2REG 0
#define OSB_RK3_LS 1
/* boundary conditions (core/boundary_conditions/periodic.py, symmetry.py, isothermal_wall.py ...) */
#define OSB_BC_PERIODIC 0
#define OSB_BC_SYMMETRY 1
#define OSB_BC_INLET_PRESSURE_EXTRAPOLATE 2 /* inlet_pressure_extrapolate.py:11-66 (x0 side 0) */
#define OSB_BC_EXTRAPOLATION 3             /* extrapolation.py:8-58, order 0 (x0 side 1) */
#define OSB_BC_ISOTHERMAL_WALL 4           /* isothermal_wall.py:11-88 (x1 side 0; side 1 on channel blocks) */
#define OSB_BC_DIRICHLET 5                 /* dirichlet.py:6-41 with a state switched at x0 (x1 side 1) */
#define OSB_BC_ADIABATIC_WALL 6            /* adiabatic_wall.py (2D: x0 faces and x1 side 0) */

/* the average the characteristic system of an interface is built from (2D blocks; 3D blocks: Roe) */
#define OSB_AVG_ROE 0    /* RoeAverage (schemes/spatial/averaging.py:62-114) */
#define OSB_AVG_SIMPLE 1 /* SimpleAverage (averaging.py:31-59): arithmetic means of rho, u_i and a */
/* one-sided closures of the central derivatives at a face of a 2D block (opensblifunctions.py:523-534) */
#define OSB_CLOSURE_REDUCED_ACCESS 0 /* reduced_access_scheme.py:6-83: first two points, 5-point stencils */
#define OSB_CLOSURE_NONE 2           /* a symmetry face of a Cartesian viscous block: central stencils
                                      * over its mirrored halos (2D) */
#define OSB_CLOSURE_CARPENTER 1      /* Carpenter_scheme.py:6-102 (every face class's default): first
                                      * derivatives at the first four points (6-point stencils), second
                                      * derivatives as ReducedAccess */
/* the WENO5 non-linear filter applied after every full time step (filters/WENO_filter.py:15-339) */
#define OSB_FILTER_NONE 0
#define OSB_FILTER_WENO5_CONSTANT 1 /* WENOFilter(block, 5, dissipation_sensor='Constant'): kappa = 1 */
/* arithmetic: all FP64 (the reference's Double datatype, core/datatypes.py:2-13), or FP32 state
 * and flux arithmetic with the RK accumulator in FP64 */
#define OSB_PREC_FP64 0
#define OSB_PREC_MIXED 1
/* reductions */
#define OSB_RED_KE 0        /* volume mean of 0.5*rho*|u|^2, FP64 */
#define OSB_RED_ENSTROPHY 1 /* volume mean of 0.5*rho*|curl u|^2, FP64, 4th-order central curl */
#define OSB_RED_NANCHECK 2  /* 1.0 if any conserved value is NaN/Inf, else 0.0 (apps/check.py:1-27) */

typedef struct osb_plan_desc {
  int abi_version;   /* OSB_ABI_VERSION */
  int ndim;          /* 3 (2 reserved for the curvilinear 2D path) */
  int n[3];          /* interior points per axis: block0np0..2 */
  double delta[3];   /* Delta0block0..2 */
  int conv, visc, rk, precision;
  int bc[3][2];      /* OSB_BC_* per axis and side */
  double gama, Minf, Re, Pr;
  double weno_eps;   /* 1e-6 in the reference's WenoJS (weno.py:341-369) */
  double teno_ct, teno_eps;
  double rk_a[3];    /* rk_sbli: rkold[]; rk_LS: A[] */
  double rk_b[3];    /* rk_sbli: rknew[]; rk_LS: B[] */
  int use_graphs;    /* capture one RK3 step as a CUDA graph */
  /* wall-bounded blocks (2D: apps/katzer_SBLI/katzer_SBLI.py; 3D with a periodic x2:
   * apps/transitional_SBLI/transitional_SBLI.py): isothermal wall temperature, Sutherland constants
   * (mu = T^1.5 (1 + SuthT/RefT)/(T + SuthT/RefT)), and the Dirichlet face's two states:
   * dirichlet_state[0] where x0 <= dirichlet_x_switch, [1] where x0 > it; the block's conserved
   * variables in order (2D: rho, rhou0, rhou1, rhoE; 3D: rho, rhou0, rhou1, rhou2, rhoE). */
  double Twall, SuthT, RefT;
  double dirichlet_state[2][5];
  double dirichlet_x_switch;
  /* TENO with the cut-off adapted per interface by the modified Ducros sensor (TENO5 on 2D blocks,
   * TENO5 or TENO6 on 3D blocks; schemes/spatial/teno.py:430-443, schemes/spatial/shock_sensors.py:
   * 12-49): at the interface whose
   * left point is P, C_T = 10^-floor(teno_a1 - teno_a2 (1 - (1 - theta)^4 (1 + 4 theta))) with
   * theta(P) = (1/2 - 1/2 tanh(2.5 + 250 div u)) (div u)^2 / (sensor_eps + (div u)^2 + |curl u|^2)
   * on the interior (0 elsewhere).  teno_adaptive = 0 keeps the fixed teno_ct. */
  int teno_adaptive;
  double teno_a1, teno_a2, sensor_eps;
  /* mixed precision on 2D blocks: an interface whose two points' pressures differ by more than this
   * factor (a strong shock) forms its Roe average, eigenvectors and characteristic reconstruction in
   * FP64 arithmetic; 0 keeps every interface in FP32.  Ignored by FP64 plans and by 3D blocks. */
  double shock_fp64;
  /* 3D wall-bounded blocks (apps/transitional_SBLI/transitional_SBLI.py): dirichlet_ke = 1 makes the
   * Dirichlet face keep rhou2 and set rhoE = dirichlet_state[.][4] + rhou2^2/(2 rho); body_force =
   * (A, xF, yF, bta, omega) adds BF = A exp(-((x0-xF)^2 + (x1-yF)^2)) cos(bta x2) sin(omega dt iter)
   * to the continuity equation, iter counting the steps the context has taken (A = 0: none). */
  int dirichlet_ke;
  double body_force[5];
  /* OSB_CLOSURE_* per axis and side of a 2D block (x0, x1; the third row is unused) */
  int closure[3][2];
  /* OSB_FILTER_*: 3D blocks with periodic or symmetry faces (no wall faces, so the filter's Wall
   * switch is 1 everywhere); filter_control is the generated code's shock_filter_control (1) */
  int filter;
  double filter_control;
  /* channel blocks (3D, periodic x0 and x2, isothermal walls on both x1 faces;
   * apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py): visc_exp is the exponent of
   * OSB_VISC_POWER; forcing = (c0, c1, c2) subtracts c_i from the momentum equations and c_j u_j from
   * the energy equation (the script's constant pressure-gradient forcing; 0: none) */
  double visc_exp;
  double forcing[3];
  /* 2D Cartesian viscous blocks (apps/viscous_shock_tube/viscous_shock_tube.py): OSB_VISC_CONST (mu = 1),
   * cartesian = 1, adiabatic walls on both x0 faces and x1 side 0, a symmetry face at x1 side 1.
   * 2D Euler blocks (OSB_VISC_NONE; apps/inviscid_shock_reflection/inviscid_shock.py): averaging is
   * OSB_AVG_*; cartesian = 1 takes x1 uniform (no metric terms; osb_set_coordinate is not called);
   * dirichlet_x0[side] is the constant state (rho, rhou0, rhou1, rhoE) of an OSB_BC_DIRICHLET x0 face.
   * Faces: x0 OSB_BC_INLET_PRESSURE_EXTRAPOLATE or OSB_BC_DIRICHLET (side 0), OSB_BC_EXTRAPOLATION or
   * OSB_BC_DIRICHLET (side 1); x1 OSB_BC_SYMMETRY (side 0), OSB_BC_DIRICHLET (switched at x0 as
   * above) or OSB_BC_SYMMETRY (side 1). */
  int averaging;
  int cartesian;
  double dirichlet_x0[2][5];
} osb_plan_desc;

/* Memory layout of every per-variable array: x fastest, interior point (i,j,k) at element
 * offset + i + j*stride_y + k*stride_z, halo depths halo[3] on both sides. */
typedef struct osb_layout {
  int64_t numel;     /* elements per variable array, halos included */
  int64_t offset;    /* element offset of interior point (0,0,0) */
  int64_t stride_y, stride_z;
  int halo[3];
  int nvar;          /* 5 in 3D */
  int state_bytes;   /* 8 (FP64) or 4 (mixed): element size of the bound state arrays */
} osb_layout;

typedef struct osb_ctx osb_ctx;

/* Validate a plan and report the layout the state arrays must have.
 * Replaces the dat declarations of defdec_data_set.h (code_generation/opsc.py:693-722). */
int osb_query_layout(const osb_plan_desc *plan, osb_layout *out);

/* Create a context; allocates the internal work arrays (second state buffer, FP64 RK register,
 * residual, reduction scratch) on the current device.  Replaces ops_init/ops_decl_* of the
 * generated main (code_generation/opsc.py:537-553). */
int osb_create(const osb_plan_desc *plan, osb_ctx **out);

/* Bind conserved variable `var` (0 rho, 1..3 rhou0..2, 4 rhoE) to a caller-owned device array of
 * the osb_query_layout layout and element size; the library never frees it. */
int osb_bind_field(osb_ctx *ctx, int var, void *dev_ptr);

/* Stream for all work of this context (cudaStream_t as void*; NULL = legacy default stream). */
int osb_set_stream(osb_ctx *ctx, void *stream);

/* Taylor-Green initial condition on the interior (apps/taylor_green_vortex/taylor_green_vortex.py:
 * 87-101, GridBasedInitialisation initialisation/gridbasedinit.py:15-57), computed in FP64 into the
 * RK register and the bound state. */
int osb_init_tgv(osb_ctx *ctx);

/* Set variable `var` from a device array that includes a halo of width h (1 <= h <= the layout's halo)
 * on every side: [n1+2h][n0+2h] in 2D, [n2+2h][n1+2h][n0+2h] in 3D, FP64.  Initial conditions whose
 * kernel also fills halos (GridBasedInitialisation ranges, initialisation/gridbasedinit.py:15-57)
 * use this. */
int osb_set_state64_padded(osb_ctx *ctx, int var, const double *dev_padded, int h);

/* 2D blocks stretched in x1: set the x1 coordinate (device FP64, [n1+2h][n0+2h] with halo h) and
 * evaluate the metric terms once: detJ = dx1/dxi1 with the boundary closures, D11 = 1/detJ with
 * mirrored halos, SD111 = dD11/dxi1 (equation_types/metric.py:37-234, 315-332). */
int osb_set_coordinate(osb_ctx *ctx, int axis, const double *dev_padded, int h);

/* Set / read the FP64 master copy of variable `var` from / into an array of n0*n1*n2 doubles laid
 * out [z][y][x] (interior only); setting also refreshes the bound state.  In FP64 mode the master copy
 * is the state itself; in mixed mode it is the FP64 RK accumulator.  The array may be device memory
 * or page-locked host memory (cudaHostAlloc / cudaHostRegister), which the kernels then read or write
 * over the host link without a staging copy; other host memory gets OSB_EINVAL.  Stream-ordered: a
 * host array must stay valid until the stream has passed the call. */
int osb_set_state64(osb_ctx *ctx, int var, const double *dev_interior);
int osb_get_state64(osb_ctx *ctx, int var, double *dev_interior);

/* Plans with teno_adaptive: evaluate the TENO cut-off C_T of the current state (after applying the
 * boundary conditions) into a device array of n0*n1 doubles laid out [x1][x0] (2D blocks) or
 * n0*n1*n2 doubles laid out [x2][x1][x0] (3D blocks).  The reference
 * stores the same field, TENO_B0, for output (StoreSome in apps/katzer_SBLI/katzer_SBLI.py);
 * values are 10^-k with k an integer. */
int osb_teno_cutoff(osb_ctx *ctx, double *dev_out);

/* Advance nsteps RK3 steps of size dt (the generated time loop, algorithm.py:440-474).  Work is
 * stream-ordered; the call returns without synchronising.  On return the bound arrays hold the
 * state with valid halos. */
int osb_step(osb_ctx *ctx, int nsteps, double dt);

/* Evaluate the spatial residual R(q) of the bound state into `var`-major device array out
 * (nvar * n0*n1*n2 values of the state precision, [var][z][y][x] interior) without advancing.
 * On 2D blocks the LS-RK register is used as scratch (its next use multiplies it by A[0] = 0). */
int osb_residual(osb_ctx *ctx, void *dev_out);

/* FP64 reduction over the interior (OSB_RED_*); synchronises the context stream. */
int osb_reduce(osb_ctx *ctx, int what, double *out);

/* Number of kernel launches the last osb_step issued (for launch accounting). */
int64_t osb_launch_count(osb_ctx *ctx);

/* Per-kernel-family timing, the GPU counterpart of OPS's ops_timing_output (opsc.py:438-439):
 * while enabled, osb_step runs without graph replay and brackets every launch with CUDA events.
 * osb_profile(ctx, 1) also clears the totals.  osb_profile_read fills up to n entries of total
 * milliseconds and launch counts for the families OSB_PF_* and returns the number of families. */
#define OSB_PF_HALO 0
#define OSB_PF_WENO_X 1
#define OSB_PF_WENO_Y 2
#define OSB_PF_WENO_Z 3
#define OSB_PF_CENTRAL_RK 4
int osb_profile(osb_ctx *ctx, int enable);
int osb_profile_read(osb_ctx *ctx, double *total_ms, int64_t *counts, int n);

/* Launch shapes of the 3D kernels.  No counterpart in the reference (the generated OPS code launches
 * every kernel with one fixed block shape).
 * WENO5-JS flux kernels: tiled, or line-marching with `seg` cells per line segment (4 <= seg <= 4096)
 * and 4 or 8 warps per block (x: each warp walks 32 y-lines; y and z: each thread walks one line,
 * 32 x-lanes by 4 or 8 lines per block).  Fused central/RK kernel: tiles of 32 x ty points (ty 8 or 16).  All shapes
 * compute the same values.  Setting a shape drops captured step graphs (re-captured at the next
 * osb_step).
 * osb_autotune times every candidate shape (`reps` launches each, CUDA events on the context
 * stream, after one warm-up launch) on the bound state, keeps the fastest, and writes the time per
 * launch in ms of the chosen shapes to best_ms[0..3] (WENO x, y, z, central; 0 for kernels the plan
 * does not use) when best_ms is not NULL.  The central kernel is timed in its residual-only form.
 * It synchronises the stream, overwrites the residual scratch (never the state or the RK register),
 * and must not be called during stream capture.  On 2D plans it does nothing and returns 0. */
#define OSB_WENO_TILE 0
#define OSB_WENO_MARCH4 1
#define OSB_WENO_MARCH8 2
#define OSB_TUNE_SLOTS 4
int osb_set_weno_shape(osb_ctx *ctx, int dir, int kind, int seg);
int osb_get_weno_shape(osb_ctx *ctx, int dir, int *kind, int *seg);
int osb_set_central_shape(osb_ctx *ctx, int ty);
/* The fused central/RK kernel of FP32 plans with WENO fluxes brings its conserved planes into shared
 * memory with TMA (cp.async.bulk.tensor, mbarrier-completed, two planes ahead).  osb_set_tma(ctx, 0)
 * selects the register-staged loads instead (same results); osb_tma_active reports 1 when the TMA
 * path serves the bound state.  A TMA wait that gives up sets a device status word, reported as
 * OSB_ETIMEOUT by the next osb_reduce. */
int osb_set_tma(osb_ctx *ctx, int enable);
int osb_tma_active(osb_ctx *ctx);
int osb_get_central_shape(osb_ctx *ctx, int *ty);
int osb_autotune(osb_ctx *ctx, int reps, double *best_ms);

/* Point probes, the counterpart of SimulationMonitor's per-point reductions
 * (core/diagnostics/simulation_monitors.py:66-108): n requests {what, i, j, k} (interior indices, k = 0
 * on 2D blocks); what = a conserved variable 0..nvar-1 or a derived quantity OSB_PROBE_*.  Values come
 * from the FP64 state (exact in both precisions) into host_out[n]; the call synchronises the stream.
 * At most OSB_PROBE_MAX requests per call. */
#define OSB_PROBE_U0 16
#define OSB_PROBE_U1 17
#define OSB_PROBE_U2 18
#define OSB_PROBE_P 19
#define OSB_PROBE_T 20
#define OSB_PROBE_MAX 4096
int osb_probe(osb_ctx *ctx, int n, const int *what_ijk, double *host_out);

/* Discrete adjoint of the time loop.  No counterpart in the reference.  FP64 3D plans with central
 * skew-symmetric or characteristic fluxes (WENO5-JS, WENO5-Z, TENO5, TENO6: differentiated through the
 * characteristic projection and the nonlinear weights; TENO weights held at the cut-off's selection)
 * and periodic boundaries (viscous terms as the plan says); other plans get OSB_EUNSUPPORTED.  Arrays are device FP64, dense interior [5][n2][n1][n0].
 * osb_adjoint_residual: out = (dR/dq)^T lam at the bound state.
 * osb_adjoint_step: lam_out = (dPhi/dq)^T lam_in, Phi = one 2-register RK3 step of size dt from the
 * bound state, whose stage states are recomputed; the bound state itself is left unchanged.
 * The first call allocates the adjoint scratch (about 57 padded fields + 15 interior fields). */
int osb_adjoint_residual(osb_ctx *ctx, const double *lam, double *out);
int osb_adjoint_step(osb_ctx *ctx, double dt, const double *lam_in, double *lam_out);

int osb_get_error(osb_ctx *ctx, char *buf, int n);
void osb_destroy(osb_ctx *ctx);

/* Batched ensembles.  No counterpart in the reference (one block per process there).  n independent
 * 3D periodic plans (central skew-symmetric or WENO5-JS fluxes, RK3, one precision for all, sizes
 * free) stepped together: per RK3 stage, one launch per halo axis and persistent tile-queue launches
 * for the WENO directions and the fused central/RK update, all instances at once; each step is one
 * CUDA graph on the batch's stream (osb_batch_set_stream).  The batch owns its device memory.
 * States are FP64 dense interior [5][n2][n1][n0] device arrays; every instance has its own dt
 * (osb_batch_set_dt, a host array of n values, before the first step).  Batches whose steps overlap
 * in time must use the same stream (the kernels share one constant-memory descriptor table).
 * osb_batch_autotune times the WENO line-marching shapes (4 or 8 lines per block, segment length)
 * and the central tile (height 8/16, z-planes per tile) over the whole batch; best_ms[0..3] (may be
 * NULL) receives the chosen shapes' times per launch (WENO x, y, z, central).  osb_batch_get_shape
 * fills out[0..7] = {kind_x, seg_x, kind_y, seg_y, kind_z, seg_z, central ty, central z-planes}.
 * More instances than the descriptor table holds give OSB_ETOOLARGE. */
typedef struct osb_batch osb_batch;
int osb_batch_create(const osb_plan_desc *plans, int n, osb_batch **out);
int osb_batch_set_stream(osb_batch *batch, void *stream);
int osb_batch_set_dt(osb_batch *batch, const double *dt);
int osb_batch_set_state64(osb_batch *batch, int inst, const double *dev_interior);
int osb_batch_get_state64(osb_batch *batch, int inst, double *dev_interior);
int osb_batch_step(osb_batch *batch, int nsteps);
int osb_batch_autotune(osb_batch *batch, int reps, double *best_ms);
int osb_batch_get_shape(osb_batch *batch, int *out, int n);
int64_t osb_batch_launch_count(osb_batch *batch);
int osb_batch_get_error(osb_batch *batch, char *buf, int n);
void osb_batch_destroy(osb_batch *batch);

/* Allocation-free variant of osb_reduce.  This entry point has no counterpart in the reference; it is
 * for callers that cannot allocate device memory where they want a diagnostic (a host framework
 * whose device memory belongs to a pool allocator, a monitoring hook between time steps).  It needs
 * no context and calls no cudaMalloc/cudaFree: the caller passes the five state arrays (layout and
 * element size of osb_query_layout for `plan`; for OSB_RED_ENSTROPHY the halos must be filled, as
 * osb_step leaves them) and `dev_out`, a device pointer to one double that receives the result
 * (stream-ordered on `stream`, no synchronisation; for OSB_RED_NANCHECK 1.0 means non-finite).
 * Its only scratch is one FP64 partial sum per z-plane in a fixed device array of
 * OSB_NOALLOC_MAX_PLANES entries, resident on every device that loads the library until exit;
 * plans with more z-planes are rejected with OSB_ETOOLARGE.  The first call on a device, with that
 * device current, looks up the array's device address; make it before any stream capture.  All
 * calls share the array: calls that overlap on the GPU race and must be serialised.  3D plans only
 * (2D plans get OSB_EUNSUPPORTED before any pointer is used); `stream` and `dev_out` must belong to
 * the current device (otherwise OSB_EINVAL), because the scratch address is that device's. */
#define OSB_NOALLOC_MAX_PLANES 2048
int osb_reduce_noalloc(const osb_plan_desc *plan, void *const fields[5], int what, double *dev_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
