/* osb_oracle.h -- CPU restatement (FP64, plain C) of OpenSBLI's generated per-timestep algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle for the GB300 backend: tests, smoke() and
 * bench.py's cpu_baseline leg may call it as the checker; the product never links or calls it.
 * It is pinned against the reference generator's own C output run here (oracle/_ref, built by
 * oracle/build_ref.py) and against committed golden fixtures (tests/golden/).
 *
 * Layout of every conserved/state array passed in or out: interior points only,
 * [var][z][y][x], x fastest; var = rho, rhou0, rhou1[, rhou2], rhoE.
 */
#ifndef OSB_ORACLE_H
#define OSB_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { OSBO_CONV_CENTRAL_SKEW = 0, OSBO_CONV_WENO5JS = 1, OSBO_CONV_TENO5 = 2, OSBO_CONV_WENO5Z = 3, OSBO_CONV_TENO6 = 4 };
enum { OSBO_VISC_NONE = 0, OSBO_VISC_CONST = 1, OSBO_VISC_SUTHERLAND = 2 };
enum { OSBO_RK3_2REG = 0, OSBO_RK3_LS_SSP = 1 };
enum { OSBO_BC_PERIODIC = 0, OSBO_BC_SYMMETRY = 1 };
/* the WENO5 non-linear filter after each full step (filters/WENO_filter.py), 3D periodic blocks */
enum { OSBO_FILTER_NONE = 0, OSBO_FILTER_WENO5_CONSTANT = 1 };

typedef struct {
  int ndim;        /* 2 or 3 */
  int n[3];        /* interior points per axis (n[2] = 1 in 2D) */
  double delta[3]; /* grid spacing per axis */
  double gama, Minf, Re, Pr;
  int conv, visc, rk;
  int bc[3][2];    /* per axis, per side */
  double teno_ct, teno_eps;
  double dt;
  int filter;             /* OSBO_FILTER_* */
  double filter_control;  /* shock_filter_control (1 in the reference) */
  /* TENO cut-off adapted by the modified Ducros sensor (teno.py:430-443, shock_sensors.py:12-49):
   * teno_adaptive = 1 with the constants a1, a2 and the sensor's epsilon; 0 keeps teno_ct */
  int teno_adaptive;
  double teno_a1, teno_a2, sensor_eps;
} osbo_cfg;

/* Taylor-Green initial condition (apps/taylor_green_vortex/taylor_green_vortex.py:87-101) on the
 * interior points, x_i = delta_i * index_i. */
int osbo_tgv_init(const osbo_cfg *cfg, double *q);

/* Advance q (interior, in/out) by nsteps RK3 steps.  ke (may be NULL) receives nsteps+1 values of
 * the volume-mean kinetic energy 0.5*rho*|u|^2 before the first and after every step. */
int osbo_run(const osbo_cfg *cfg, double *q, int nsteps, double *ke);

/* One residual evaluation R(q) on the interior (the right-hand side of one RK stage), for
 * kernel-level parity tests.  r has the same layout as q. */
int osbo_residual(const osbo_cfg *cfg, const double *q, double *r);
/* adaptive TENO plans: the cut-off C_T at every interior point of the state q (after the boundary
 * conditions), laid out like one variable of q (the reference's TENO_B0 field) */
int osbo_cutoff(const osbo_cfg *cfg, const double *q, double *ct);

/* ---- 2D curvilinear shock/boundary-layer path (TENO5, metrics, Sutherland, walls, LS-RK3) ---- */
typedef struct {
  int n[2];          /* interior points in x0, x1 */
  double delta[2];   /* computational spacing: Delta0block0, Delta1block0 */
  double gama, Minf, Re, Pr, Twall, SuthT, RefT;
  double teno_eps, teno_ct;
  double Lx1, by;    /* x1 = Lx1 sinh(by delta1 j / Lx1) / sinh(by) */
  double rkA[3], rkB[3];
  double dt;
  /* adaptive TENO (teno.py:430-443) driven by the modified Ducros sensor (shock_sensors.py:12-49):
   * C_T = 10^-floor(a1 - a2 (1 - (1-theta)^4 (1+4 theta))) per interface; 0 selects the fixed teno_ct */
  int teno_adaptive;
  double teno_a1, teno_a2, sensor_eps;
  /* one-sided closure of the central first derivatives at each face [axis][side]:
   * 0 ReducedAccess (reduced_access_scheme.py), 1 Carpenter (Carpenter_scheme.py) */
  int closure[2][2];
  /* characteristic scheme: OSBO_CONV_TENO5 (default 0 is read as TENO5), OSBO_CONV_WENO5JS,
   * OSBO_CONV_WENO5Z or OSBO_CONV_TENO6 */
  int conv;
  /* 2D Euler blocks (apps/inviscid_shock_reflection/inviscid_shock.py): euler = 1 drops the viscous
   * terms and the metric (x1 uniform, D11 = 1).  bc[axis][side]: OSBO_BC2_DEFAULT (the shock/boundary-
   * layer face of that side: inlet, extrapolation, isothermal wall, the script's Dirichlet top),
   * OSBO_BC2_DIRICHLET or OSBO_BC2_SYMMETRY; face0[side] is the constant state of a Dirichlet x0
   * face, top[0] / top[1] the states of a Dirichlet x1 side-1 face where x0 <= x_switch / x0 >
   * x_switch (rho, rhou0, rhou1, rhoE).  simple_avg = 1: the characteristic system at an interface
   * from the arithmetic means of rho, u and a (SimpleAverage, averaging.py:31-59). */
  int euler, simple_avg;
  int bc[2][2];
  double face0[2][4], top[2][4], x_switch;
  /* rk2reg = 1: RungeKutta(3) with two registers (rk_sbli.py:51-61, 117-124): at the step's start
   * qold = q; per stage q = qold + rkB dt R, then qold += rkA dt R (rkA = rkold, rkB = rknew) */
  int rk2reg;
  /* Cartesian viscous blocks (apps/viscous_shock_tube/viscous_shock_tube.py): cartesian = 1 takes D11 = 1
   * with the viscous terms kept; visc_const = 1 takes mu = 1 (the script's constant mu) */
  int cartesian, visc_const;
  /* the laminar channel (apps/channel_flow/laminar_2D/laminar_channel.py): skew = 1 takes the central
   * skew-symmetric convective terms instead of the characteristic fluxes, force = c_j subtracted from the
   * momentum (c_i) and energy (c_j u_j) equations */
  int skew;
  double force[2];
} osbo2d_cfg;
#define OSBO_BC2_DEFAULT 0
#define OSBO_BC2_DIRICHLET 1
#define OSBO_BC2_SYMMETRY 2
#define OSBO_BC2_PERIODIC 3 /* periodic.py / exchange.py:9-57 (both sides of the axis) */
#define OSBO_BC2_ADIABATIC 4 /* adiabatic_wall.py: no slip, zero wall-normal temperature gradient */
#define OSBO_BC2_WALL 5      /* isothermal_wall.py on x1 side 1 (the channel's second wall) */

/* Advance q by nsteps LS-RK3 steps.  q holds [4][n1+8][n0+8]: rho, rhou0, rhou1, rhoE with a
 * 4-point halo on every side (the initial state must fill the halos as the script's
 * initialisation kernel does); it is overwritten with the final state, halos included. */
int osbo2d_run(const osbo2d_cfg *cfg, double *q, int nsteps);
/* The right-hand side of q (boundary conditions applied first) on the interior, [4][n1][n0]. */
int osbo2d_residual(const osbo2d_cfg *cfg, const double *q, double *r);
/* ---- 1D Euler blocks (apps/Sod_shock_tube, apps/shu_osher) ---- */
typedef struct {
  int n0;
  double delta0, gama;
  int conv;          /* OSBO_CONV_TENO5 (0), OSBO_CONV_WENO5JS, OSBO_CONV_WENO5Z, OSBO_CONV_TENO6 */
  double teno_eps, teno_ct;
  int simple_avg;    /* 1: SimpleAverage, 0: RoeAverage */
  double rkA[3], rkB[3];
  double dt;
  int bc1;           /* side 1: 0 Dirichlet (face[1]), 1 extrapolation; side 0 is Dirichlet (face[0]) */
  double face[2][3]; /* rho, rhou0, rhoE */
} osbo1d_cfg;
/* Advance q [3][n0+8] (4-point halo) by nsteps LS-RK3 steps, in place. */
int osbo1d_run(const osbo1d_cfg *cfg, double *q, int nsteps);
/* The right-hand side [3][n0] of q (boundary conditions applied first). */
int osbo1d_residual(const osbo1d_cfg *cfg, const double *q, double *r);
/* ---- 3D span-periodic wall-bounded path: the 2D configuration above with a periodic x2 axis ---- */
typedef struct {
  int n[3];          /* interior points in x0, x1, x2 */
  double delta[3];   /* computational spacing: Delta0block0, Delta1block0, Delta2block0 */
  double gama, Minf, Re, Pr, Twall, SuthT, RefT;
  double teno_eps, teno_ct;
  double Lx1, by;    /* x1 = Lx1 sinh(by delta1 j / Lx1) / sinh(by) */
  double rkA[3], rkB[3];
  double dt;
  int closure[2][2]; /* [axis 0, 1][side]: 0 ReducedAccess, 1 Carpenter */
  int conv;          /* OSBO_CONV_TENO5 (0 read as TENO5), OSBO_CONV_WENO5JS, OSBO_CONV_WENO5Z, OSBO_CONV_TENO6 */
  /* Dirichlet face (x1 side 1): state[1] where x0 = delta0 i > x_switch, state[0] elsewhere;
   * rho, rhou0, rhou1, rhou2, rhoE */
  double dirichlet[2][5];
  double x_switch;
  /* dirichlet_ke = 1: the Dirichlet face keeps rhou2 and sets rhoE = dirichlet[.][4] + rhou2^2/(2 rho)
   * with the face's rho (apps/transitional_SBLI/transitional_SBLI.py:110-116) */
  int dirichlet_ke;
  /* body force in the continuity equation (transitional_SBLI.py:80-89), 0 when bf_A = 0:
   * BF = bf_A exp(-((x0-bf_xF)^2 + (x1-bf_yF)^2)) cos(bf_bta x2) sin(bf_omega dt iter) */
  double bf_A, bf_xF, bf_yF, bf_bta, bf_omega;
  /* TENO cut-off adapted by the metric-transformed Ducros sensor (0: the fixed teno_ct) */
  int teno_adaptive;
  double teno_a1, teno_a2, sensor_eps;
  /* channel blocks (apps/channel_flow/compressible_TCF_TENO/turbulent_channel.py): periodic0 = 1
   * makes x0 periodic (no inlet or outlet face), wall1 = 1 puts an isothermal wall on x1 side 1 (no
   * Dirichlet face), grid_tanh = 1 takes x1 = -tanh(stretch (1 - 2 j/(n1-1))) / tanh(stretch),
   * visc_pow > 0 takes mu = T^visc_pow (0: Sutherland), force = c_j of the momentum (-c_i) and energy
   * (-c_j u_j) equations */
  int periodic0, wall1, grid_tanh;
  double stretch, visc_pow;
  double force[3];
} osbo3w_cfg;

/* Advance q by nsteps LS-RK3 steps.  q holds [5][n2+8][n1+8][n0+8] with a 4-point halo on every side
 * (the initial state fills the halos as the script's initialisation kernel does); it is overwritten
 * with the final state, halos included. */
int osbo3w_run(const osbo3w_cfg *cfg, double *q, int nsteps);
/* The right-hand side of q (boundary conditions applied first) on the interior, [5][n2][n1][n0]. */
int osbo3w_residual(const osbo3w_cfg *cfg, const double *q, double *r);

/* Metric terms D11 and SD111 on the interior, [n1][n0]. */
int osbo2d_cutoff(const osbo2d_cfg *cfg, const double *q, double *ct);
int osbo2d_metrics(const osbo2d_cfg *cfg, double *D11, double *SD111);
/* The Carpenter first-derivative closure weights, [4][6] row-major: weight of f(m) at point r. */
void osbo2d_carpenter_d1(double *c24);

#ifdef __cplusplus
}
#endif
#endif
