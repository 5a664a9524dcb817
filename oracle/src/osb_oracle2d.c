/* osb_oracle2d.c -- CPU restatement (FP64) of the generated per-timestep algorithm for the 2D
 * curvilinear shock/boundary-layer configuration (TENO5, metrics, isothermal wall).
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle).  See osb_oracle.h.
 *
 * The kernel list restated here is the one TraditionalAlgorithmRK builds for a block with
 * MetricsEquation (stretched in x1), LLFTeno(5), Central(4), Sutherland viscosity, RungeKuttaLS(3,'SSP')
 * and the four boundary conditions InletPressureExtrapolateBC / ExtrapolationBC (x) and
 * IsothermalWallBC / DirichletBC (y), each face with the ReducedAccess or the Carpenter closure
 * (apps/katzer_SBLI/katzer_SBLI.py:32-126 with fixed-C_T TENO).  Order (algorithm.py:384-477):
 *   before the loop: coordinates, metric derivative, D11 = 1/(dx1/dxi1), metric halos, SD111
 *   iter { BCs; stage { CRs; TENO x; TENO y; TENO residual; viscous terms; LS-RK update; BCs } }
 * Arrays carry a 5-point halo.  The state exchanged with callers carries a 4-point halo.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "osb_oracle.h"

#define H 5

/* the 3D restatement's reconstruction sides (osb_oracle.c) */
double osbo_side_weno5_plus(const double f[5], int z);
double osbo_side_weno5_minus(const double g[5], int z);
double osbo_side_teno6(const double g[6], int plus, double eps, double CT);

typedef struct {
  osbo2d_cfg c;
  int px, py;
  size_t np;
  double *q[4], *du[4], *res[4];
  double *u0, *u1, *p, *a, *T, *mu, *theta;
  double *x1, *D11, *SD111, *flux[4];
  double carp[4][6]; /* Carpenter first-derivative closure weights */
} s2_t;

static inline size_t I2(const s2_t *s, int i, int j) { return (size_t)(i + H) + (size_t)s->px * (size_t)(j + H); }
static double *alloc2(const s2_t *s) { return (double *)calloc(s->np, sizeof(double)); }

#define N0 (s->c.n[0])
#define N1 (s->c.n[1])
#define FOR2(i0, i1, j0, j1) for (int j = (j0); j < (j1); ++j) for (int i = (i0); i < (i1); ++i)

static void carpenter_d1(double c[4][6]);

static void s2_init(s2_t *s, const osbo2d_cfg *cfg) {
  memset(s, 0, sizeof(*s));
  s->c = *cfg;
  carpenter_d1(s->carp);
  s->px = cfg->n[0] + 2 * H;
  s->py = cfg->n[1] + 2 * H;
  s->np = (size_t)s->px * s->py;
  for (int v = 0; v < 4; ++v) {
    s->q[v] = alloc2(s);
    s->du[v] = alloc2(s);
    s->res[v] = alloc2(s);
    s->flux[v] = alloc2(s);
  }
  s->u0 = alloc2(s); s->u1 = alloc2(s); s->p = alloc2(s); s->a = alloc2(s); s->T = alloc2(s); s->mu = alloc2(s);
  s->theta = alloc2(s); /* written on the interior only; the rest stays 0, as the generated code leaves it */
  s->x1 = alloc2(s); s->D11 = alloc2(s); s->SD111 = alloc2(s);
}

static void s2_free(s2_t *s) {
  for (int v = 0; v < 4; ++v) { free(s->q[v]); free(s->du[v]); free(s->res[v]); free(s->flux[v]); }
  free(s->u0); free(s->u1); free(s->p); free(s->a); free(s->T); free(s->mu); free(s->theta);
  free(s->x1); free(s->D11); free(s->SD111);
}

/* ---------------------------------------------------------------------------------------------
 * 4th-order central derivatives in computational space with one-sided closures at the faces
 * (applied through opensblifunctions.py:523-534):
 *  - ReducedAccess (core/boundary_conditions/reduced_access_scheme.py:34-83): first and second
 *    derivatives at the first two and last two points, 5-point stencils;
 *  - Carpenter (core/boundary_conditions/Carpenter_scheme.py:6-102, after the paper it cites,
 *    doi:10.1006/jcph.1998.6114): first derivatives at the first four points from the 4x6 matrix
 *    A^-1 B of the published boundary closure (free parameters R1, R2 as in the reference), mirrored
 *    with the opposite sign on side 1; the second derivative uses the same two-point closure as
 *    ReducedAccess.
 * ------------------------------------------------------------------------------------------- */
static inline double F(const s2_t *s, const double *f, int i, int j) { return f[I2(s, i, j)]; }

/* c[r][m]: weight of f(m) in the first derivative at point r of a side-0 face */
static void carpenter_d1(double c[4][6]) {
  const double R1 = -(2177.0 * sqrt(295369.0) - 1166427.0) / 25488.0;
  const double R2 = (66195.0 * sqrt(53.0) * sqrt(5573.0) - 35909375.0) / 101952.0;
  const double P = 216.0 * R2 + 2160.0 * R1, Q = 81.0 * R2 + 675.0 * R1, S = 864.0 * R2 + 6480.0 * R1;
  /* A: the norm-matrix block of the closure (symmetric), B: the difference-operator block */
  double A[4][10] = {
      {-(P - 2125.0) / 12960.0, (Q + 415.0) / 540.0, -(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0,
       -(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0},
      {(Q + 415.0) / 540.0, -(4104.0 * R2 + 32400.0 * R1 + 11225.0) / 4320.0,
       (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0, -(P + 655.0) / 4320.0},
      {-(72.0 * R2 + 720.0 * R1 + 445.0) / 1440.0, (1836.0 * R2 + 14580.0 * R1 + 7295.0) / 2160.0,
       -(4104.0 * R2 + 32400.0 * R1 + 12785.0) / 4320.0, (Q + 335.0) / 540.0},
      {-(108.0 * R2 + 756.0 * R1 + 421.0) / 1296.0, -(P + 655.0) / 4320.0, (Q + 335.0) / 540.0,
       -(P - 12085.0) / 12960.0}};
  const double B[4][6] = {
      {-0.5, -(S + 305.0) / 4320.0, (216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0, -(S + 3335.0) / 4320.0, 0.0, 0.0},
      {(S + 305.0) / 4320.0, 0.0, -(S + 2315.0) / 1440.0, (108.0 * R2 + 810.0 * R1 + 415.0) / 270.0, 0.0, 0.0},
      {-(216.0 * R2 + 1620.0 * R1 + 725.0) / 540.0, (S + 2315.0) / 1440.0, 0.0, -(S + 785.0) / 4320.0, -1.0 / 12.0,
       0.0},
      {(S + 3335.0) / 4320.0, -(108.0 * R2 + 810.0 * R1 + 415.0) / 270.0, (S + 785.0) / 4320.0, 0.0, 8.0 / 12.0,
       -1.0 / 12.0}};
  /* Gauss-Jordan elimination with partial pivoting on [A | B] */
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) A[r][4 + m] = B[r][m];
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
    for (int m = 0; m < 10; ++m) {
      const double t = A[col][m];
      A[col][m] = A[piv][m];
      A[piv][m] = t;
    }
    const double inv = 1.0 / A[col][col];
    for (int m = 0; m < 10; ++m) A[col][m] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const double f = A[r][col];
      for (int m = 0; m < 10; ++m) A[r][m] -= f * A[col][m];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) c[r][m] = A[r][4 + m];
}

static double d1c(const s2_t *s, const double *f, int i, int j, int dir) {
  const int n = dir == 0 ? N0 : N1, k = dir == 0 ? i : j;
  const double inv = 1.0 / s->c.delta[dir];
  const int c0 = s->c.closure[dir][0], c1 = s->c.closure[dir][1];
#define G(o) (dir == 0 ? F(s, f, i + (o), j) : F(s, f, i, j + (o)))
  /* the side-0 face's points take precedence (its condition comes first in the Piecewise) */
  /* closure 2: none (a symmetry face, whose mirrored halos the central stencil reads) */
  int side = -1, r = 0;
  if (k < (c0 == 1 ? 4 : c0 == 2 ? 0 : 2)) side = 0, r = k;
  else if (n - 1 - k < (c1 == 1 ? 4 : c1 == 2 ? 0 : 2)) side = 1, r = n - 1 - k;
  const int carp = side >= 0 && (side == 0 ? c0 : c1) == 1;
  double v;
  if (carp) {
    /* side 0: point r reads f(0..5); side 1: point n-1-r reads f(n-1-m), sign reversed */
    v = 0.0;
    for (int m = 0; m < 6; ++m) v += s->carp[r][m] * (side == 0 ? G(m - r) : G(r - m));
    if (side == 1) v = -v;
  } else if (side == 0 && r == 0) v = -(25.0 / 12.0) * G(0) + 4.0 * G(1) - 3.0 * G(2) + (4.0 / 3.0) * G(3) - 0.25 * G(4);
  else if (side == 0) v = -0.25 * G(-1) - (5.0 / 6.0) * G(0) + 1.5 * G(1) - 0.5 * G(2) + (1.0 / 12.0) * G(3);
  else if (side == 1 && r == 0) v = (25.0 / 12.0) * G(0) - 4.0 * G(-1) + 3.0 * G(-2) - (4.0 / 3.0) * G(-3) + 0.25 * G(-4);
  else if (side == 1) v = 0.25 * G(1) + (5.0 / 6.0) * G(0) - 1.5 * G(-1) + 0.5 * G(-2) - (1.0 / 12.0) * G(-3);
  else v = (1.0 / 12.0) * G(-2) - (2.0 / 3.0) * G(-1) + (2.0 / 3.0) * G(1) - (1.0 / 12.0) * G(2);
#undef G
  return inv * v;
}

/* coefficient table of the Carpenter first-derivative closure (for the tests) */
void osbo2d_carpenter_d1(double *c24) {
  double c[4][6];
  carpenter_d1(c);
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) c24[6 * r + m] = c[r][m];
}

static double d2c(const s2_t *s, const double *f, int i, int j, int dir) {
  const int n = dir == 0 ? N0 : N1, k = dir == 0 ? i : j;
  const double inv = 1.0 / (s->c.delta[dir] * s->c.delta[dir]);
#define G(o) (dir == 0 ? F(s, f, i + (o), j) : F(s, f, i, j + (o)))
  double v;
  const int open0 = s->c.closure[dir][0] != 2, open1 = s->c.closure[dir][1] != 2; /* 2: no closure */
  if (k == 0 && open0)
    v = (35.0 / 12.0) * G(0) - (26.0 / 3.0) * G(1) + 9.5 * G(2) - (14.0 / 3.0) * G(3) + (11.0 / 12.0) * G(4);
  else if (k == 1 && open0)
    v = (11.0 / 12.0) * G(-1) - (5.0 / 3.0) * G(0) + 0.5 * G(1) + (1.0 / 3.0) * G(2) - (1.0 / 12.0) * G(3);
  else if (k == n - 1 && open1)
    v = (35.0 / 12.0) * G(0) - (26.0 / 3.0) * G(-1) + 9.5 * G(-2) - (14.0 / 3.0) * G(-3) + (11.0 / 12.0) * G(-4);
  else if (k == n - 2 && open1)
    v = (11.0 / 12.0) * G(1) - (5.0 / 3.0) * G(0) + 0.5 * G(-1) + (1.0 / 3.0) * G(-2) - (1.0 / 12.0) * G(-3);
  else
    v = -(1.0 / 12.0) * G(-2) + (4.0 / 3.0) * G(-1) - 2.5 * G(0) + (4.0 / 3.0) * G(1) - (1.0 / 12.0) * G(2);
#undef G
  return inv * v;
}

/* ---------------------------------------------------------------------------------------------
 * Metrics (equation_types/metric.py:37-234, 315-332), grid stretched in x1 only:
 *   x1(j) = Lx1 sinh(by delta1 j / Lx1) / sinh(by)   (the script's coordinate equation)
 *   detJ = dx1/dxi1, D11 = 1/detJ, halos mirrored about the boundary points, SD111 = dD11/dxi1.
 * ------------------------------------------------------------------------------------------- */
static void metrics(s2_t *s) {
  if (s->c.euler || s->c.cartesian) { /* no metric kernels in a Cartesian block: d/dx1 = d/dxi1 */
    FOR2(-H, N0 + H, -H, N1 + H) {
      s->D11[I2(s, i, j)] = 1.0;
      s->SD111[I2(s, i, j)] = 0.0;
    }
    return;
  }
  const double Lx1 = s->c.Lx1, by = s->c.by, d1 = s->c.delta[1];
  FOR2(-3, N0 + 4, -3, N1 + 4) s->x1[I2(s, i, j)] = sinh(d1 * by * (1.0 / Lx1) * j) / ((1.0 / Lx1) * sinh(by));
  double *wk = alloc2(s);
  FOR2(0, N0, 0, N1) wk[I2(s, i, j)] = d1c(s, s->x1, i, j, 1);
  FOR2(0, N0, 0, N1) s->D11[I2(s, i, j)] = 1.0 / wk[I2(s, i, j)];
  /* metric boundary kernels: dir0 side0, dir0 side1, dir1 side0, dir1 side1 */
  for (int j = -3; j < N1 + 4; ++j)
    for (int t = 1; t <= 3; ++t) s->D11[I2(s, -t, j)] = s->D11[I2(s, t, j)];
  for (int j = -3; j < N1 + 4; ++j)
    for (int t = 1; t <= 4; ++t) s->D11[I2(s, N0 - 1 + t, j)] = s->D11[I2(s, N0 - 1 - t, j)];
  for (int i = -3; i < N0 + 4; ++i)
    for (int t = 1; t <= 3; ++t) s->D11[I2(s, i, -t)] = s->D11[I2(s, i, t)];
  for (int i = -3; i < N0 + 4; ++i)
    for (int t = 1; t <= 4; ++t) s->D11[I2(s, i, N1 - 1 + t)] = s->D11[I2(s, i, N1 - 1 - t)];
  FOR2(0, N0, 0, N1) s->SD111[I2(s, i, j)] = d1c(s, s->D11, i, j, 1);
  free(wk);
}

/* ---------------------------------------------------------------------------------------------
 * Boundary conditions, applied in the order x0 side0, x0 side1, x1 side0, x1 side1.
 * ------------------------------------------------------------------------------------------- */
/* InletPressureExtrapolateBC (core/boundary_conditions/inlet_pressure_extrapolate.py:11-66): at
 * i = 0, supersonic points take the halo state at i = -1; subsonic points keep theirs and the
 * energy halos take rhoE(0). */
static void bc_inlet(s2_t *s) {
  const double g = s->c.gama;
  for (int j = -3; j < N1 + 4; ++j) {
    const size_t b = I2(s, 0, j);
    const double rhob = s->q[0][b];
    const double ub0 = fabs(s->q[1][b] / rhob), ub1 = fabs(s->q[2][b] / rhob);
    const double pb = (g - 1) * (-0.5 * rhob * (ub0 * ub0 + ub1 * ub1) + s->q[3][b]);
    const double ab = sqrt(g * pb / rhob);
    if (ub0 >= ab) {
      for (int v = 0; v < 4; ++v) s->q[v][b] = s->q[v][I2(s, -1, j)];
    } else {
      for (int t = 1; t <= 3; ++t) s->q[3][I2(s, -t, j)] = s->q[3][b];
    }
  }
}

/* ExtrapolationBC order 0 (core/boundary_conditions/extrapolation.py:8-58): the last point and the
 * halo take the state of point n-2. */
static void bc_outlet(s2_t *s) {
  for (int j = -3; j < N1 + 4; ++j)
    for (int v = 0; v < 4; ++v) {
      const double val = s->q[v][I2(s, N0 - 2, j)];
      for (int t = 0; t <= 4; ++t) s->q[v][I2(s, N0 - 1 + t, j)] = val;
    }
}

/* IsothermalWallBC (core/boundary_conditions/isothermal_wall.py:32-88): no slip and
 * rhoE = rho Twall/(gama (gama-1) Minf^2) at the wall; halo t gets T_t = (t+1) Twall - t T_above,
 * rho_t = gama Minf^2 Pwall / T_t, momentum of the mirror point reversed, energy from Pwall. */
static void bc_wall(s2_t *s) {
  const double g = s->c.gama, M = s->c.Minf, Tw = s->c.Twall;
  for (int i = -3; i < N0 + 4; ++i) {
    const size_t w = I2(s, i, 0);
    s->q[1][w] = 0.0;
    s->q[2][w] = 0.0;
    s->q[3][w] = Tw * (1.0 / (M * M)) * s->q[0][w] / (g * (g - 1.0));
    const double Pw = (g - 1) * (-(0.5 * s->q[1][w] * s->q[1][w] + 0.5 * s->q[2][w] * s->q[2][w]) / s->q[0][w] + s->q[3][w]);
    const size_t a1 = I2(s, i, 1);
    const double Ta = M * M * g * (g - 1) *
                      (-(0.5 * s->q[1][a1] * s->q[1][a1] + 0.5 * s->q[2][a1] * s->q[2][a1]) / s->q[0][a1] + s->q[3][a1]) /
                      s->q[0][a1];
    for (int t = 1; t <= 3; ++t) {
      const size_t m = I2(s, i, t), h = I2(s, i, -t);
      const double um0 = s->q[1][m] / s->q[0][m], um1 = s->q[2][m] / s->q[0][m];
      const double Tt = (t + 1) * Tw - t * Ta;
      const double rh = M * M * g * Pw / Tt;
      s->q[0][h] = rh;
      s->q[1][h] = -rh * um0;
      s->q[2][h] = -rh * um1;
      s->q[3][h] = (1.0 / (g - 1)) * Pw + 0.5 * rh * (um0 * um0 + um1 * um1);
    }
  }
}

/* DirichletBC with the shock generator of the script (katzer_SBLI.py:108-114): points j >= n1-1 take
 * the post-shock state where x0 > 40, the pre-shock state elsewhere. */
static void bc_top(s2_t *s) {
  static const double post[4] = {1.129734572, 1.0921171, -0.058866065, 1.0590824};
  static const double pre[4] = {1.00000596004, 1.00000268202, 0.00565001630205, 0.94644428042};
  for (int j = N1 - 1; j < N1 + 4; ++j)
    for (int i = -3; i < N0 + 4; ++i) {
      const double x0 = s->c.delta[0] * i;
      for (int v = 0; v < 4; ++v) s->q[v][I2(s, i, j)] = x0 > 40.0 ? post[v] : pre[v];
    }
}

/* DirichletBC on an x0 face (dirichlet.py:6-41): the boundary point and the halo take the constant
 * state of the face (side 0: i = -3..0; side 1: i = n0-1..n0+3). */
static void bc_dirichlet_x0(s2_t *s, int side) {
  const double *st = s->c.face0[side];
  const int i0 = side == 0 ? -3 : N0 - 1, i1 = side == 0 ? 1 : N0 + 4;
  for (int j = -3; j < N1 + 4; ++j)
    for (int i = i0; i < i1; ++i)
      for (int v = 0; v < 4; ++v) s->q[v][I2(s, i, j)] = st[v];
}

/* SymmetryBC on an x1 face (symmetry.py): halo point t mirrors the interior point t away from the
 * boundary point, the normal momentum reversed; the boundary point keeps its values. */
static void bc_symmetry_x1(s2_t *s, int side) {
  const int jb = side == 0 ? 0 : N1 - 1, sg = side == 0 ? 1 : -1, nt = side == 0 ? 3 : 4;
  for (int i = -3; i < N0 + 4; ++i)
    for (int t = 1; t <= nt; ++t) {
      const size_t h = I2(s, i, jb - sg * t), m = I2(s, i, jb + sg * t);
      for (int v = 0; v < 4; ++v) s->q[v][h] = v == 2 ? -s->q[v][m] : s->q[v][m];
    }
}

/* DirichletBC on x1 side 1 with a state switched at x0 (the shock generator of an Euler block) */
static void bc_top_states(s2_t *s) {
  for (int j = N1 - 1; j < N1 + 4; ++j)
    for (int i = -3; i < N0 + 4; ++i) {
      const double x0 = s->c.delta[0] * i;
      for (int v = 0; v < 4; ++v) s->q[v][I2(s, i, j)] = s->c.top[x0 > s->c.x_switch ? 1 : 0][v];
    }
}

/* The periodic exchange of axis d (exchange.py:9-57): the halo points take the interior points one
 * period away, every row (column) of the padded block. */
static void bc_periodic(s2_t *s, int d) {
  for (int v = 0; v < 4; ++v)
    for (int a = -H; a < (d == 0 ? N1 : N0) + H; ++a)
      for (int t = 1; t <= H; ++t) {
        if (d == 0) {
          s->q[v][I2(s, -t, a)] = s->q[v][I2(s, N0 - t, a)];
          s->q[v][I2(s, N0 - 1 + t, a)] = s->q[v][I2(s, t - 1, a)];
        } else {
          s->q[v][I2(s, a, -t)] = s->q[v][I2(s, a, N1 - t)];
          s->q[v][I2(s, a, N1 - 1 + t)] = s->q[v][I2(s, a, t - 1)];
        }
      }
}

/* AdiabaticWallBC (adiabatic_wall.py, as generated for viscous_shock_tube.py) on the face of axis d,
 * side `side`, every line across it: zero momentum at the wall point, the wall temperature from the
 * one-sided zero-gradient formula T_w = (18 T_1 - 9 T_2 + 2 T_3)/11 over the first three interior
 * points and rhoE_w = rho_w T_w / (gama Minf^2 (gama-1)); halo point t mirrors interior point t with
 * rho and rhoE even and the momentum odd (t = 1..3 on side 0, 1..4 on side 1). */
static void bc_adiabatic(s2_t *s, int d, int side) {
  const double g = s->c.gama, M2 = s->c.Minf * s->c.Minf;
  const int n = d == 0 ? N0 : N1, len = d == 0 ? N1 : N0, bnd = side == 0 ? 0 : n - 1;
  const int sg = side == 0 ? 1 : -1, nt = side == 0 ? 3 : 4;
  for (int a = -3; a < len + 4; ++a) {
#define AT(k) (d == 0 ? I2(s, (k), a) : I2(s, a, (k)))
    for (int t = 1; t <= nt; ++t) s->q[0][AT(bnd - sg * t)] = s->q[0][AT(bnd + sg * t)];
    s->q[1][AT(bnd)] = 0.0;
    s->q[2][AT(bnd)] = 0.0;
    for (int t = 1; t <= nt; ++t)
      for (int v = 1; v <= 2; ++v) s->q[v][AT(bnd - sg * t)] = -s->q[v][AT(bnd + sg * t)];
    double T[4];
    for (int k = 1; k <= 3; ++k) {
      const size_t m = AT(bnd + sg * k);
      const double p = (g - 1) * (s->q[3][m] - 0.5 * (s->q[1][m] * s->q[1][m] + s->q[2][m] * s->q[2][m]) / s->q[0][m]);
      T[k] = g * M2 * p / s->q[0][m];
    }
    s->q[3][AT(bnd)] = (18.0 / 11.0 * T[1] - 9.0 / 11.0 * T[2] + 2.0 / 11.0 * T[3]) * s->q[0][AT(bnd)] / (g * M2 * (g - 1));
    for (int t = 1; t <= nt; ++t) s->q[3][AT(bnd - sg * t)] = s->q[3][AT(bnd + sg * t)];
#undef AT
  }
}

/* IsothermalWallBC on x1 side 1 (isothermal_wall.py:32-88): bc_wall mirrored about row n1-1, halo
 * rows n1..n1+3 */
static void bc_wall_top(s2_t *s) {
  const double g = s->c.gama, M = s->c.Minf, Tw = s->c.Twall;
  const int jw = N1 - 1;
  for (int i = -3; i < N0 + 4; ++i) {
    const size_t w = I2(s, i, jw), a1 = I2(s, i, jw - 1);
    s->q[1][w] = 0.0;
    s->q[2][w] = 0.0;
    s->q[3][w] = Tw * (1.0 / (M * M)) * s->q[0][w] / (g * (g - 1.0));
    const double Pw = (g - 1) * s->q[3][w];
    const double Ta = M * M * g * (g - 1) *
                      (-(0.5 * s->q[1][a1] * s->q[1][a1] + 0.5 * s->q[2][a1] * s->q[2][a1]) / s->q[0][a1] + s->q[3][a1]) /
                      s->q[0][a1];
    for (int t = 1; t <= 4; ++t) {
      const size_t m = I2(s, i, jw - t), h = I2(s, i, jw + t);
      const double um0 = s->q[1][m] / s->q[0][m], um1 = s->q[2][m] / s->q[0][m];
      const double Tt = (t + 1) * Tw - t * Ta;
      const double rh = M * M * g * Pw / Tt;
      s->q[0][h] = rh;
      s->q[1][h] = -rh * um0;
      s->q[2][h] = -rh * um1;
      s->q[3][h] = (1.0 / (g - 1)) * Pw + 0.5 * rh * (um0 * um0 + um1 * um1);
    }
  }
}

static void apply_bcs(s2_t *s) {
  const int(*b)[2] = s->c.bc;
  if (b[0][0] == OSBO_BC2_PERIODIC && b[1][0] != OSBO_BC2_PERIODIC) { /* laminar_channel.py */
    bc_periodic(s, 0);
    bc_wall(s);
    bc_wall_top(s);
    return;
  }
  if (b[0][0] == OSBO_BC2_ADIABATIC) { /* viscous_shock_tube.py: adiabatic walls and a symmetry top */
    bc_adiabatic(s, 0, 0);
    bc_adiabatic(s, 0, 1);
    bc_adiabatic(s, 1, 0);
    bc_symmetry_x1(s, 1);
    return;
  }
  if (b[0][0] == OSBO_BC2_PERIODIC) { /* a doubly periodic Euler block (euler_wave.py) */
    bc_periodic(s, 0);
    bc_periodic(s, 1);
    return;
  }
  if (b[0][0] == OSBO_BC2_DIRICHLET) bc_dirichlet_x0(s, 0);
  else bc_inlet(s);
  if (b[0][1] == OSBO_BC2_DIRICHLET) bc_dirichlet_x0(s, 1);
  else bc_outlet(s);
  if (b[1][0] == OSBO_BC2_SYMMETRY) bc_symmetry_x1(s, 0);
  else bc_wall(s);
  if (b[1][1] == OSBO_BC2_SYMMETRY) bc_symmetry_x1(s, 1);
  else if (b[1][1] == OSBO_BC2_DIRICHLET) bc_top_states(s);
  else bc_top(s);
}

/* ---------------------------------------------------------------------------------------------
 * Constituent relations (katzer_SBLI.py:17-22): u_i, p, a over -3..n+4; T, mu (Sutherland) over
 * -2..n+2.
 * ------------------------------------------------------------------------------------------- */
static void constituent(s2_t *s) {
  const double g = s->c.gama, M = s->c.Minf, ST = s->c.SuthT / s->c.RefT;
  FOR2(-3, N0 + 4, -3, N1 + 4) {
    const size_t n = I2(s, i, j);
    const double r = s->q[0][n];
    const double u0 = s->q[1][n] / r, u1 = s->q[2][n] / r;
    s->u0[n] = u0;
    s->u1[n] = u1;
    s->p[n] = (g - 1) * (s->q[3][n] - 0.5 * r * u0 * u0 - 0.5 * r * u1 * u1);
    s->a[n] = sqrt(g * s->p[n] / r);
  }
  FOR2(-2, N0 + 2, -2, N1 + 2) {
    const size_t n = I2(s, i, j);
    s->T[n] = M * M * g * s->p[n] / s->q[0][n];
    s->mu[n] = s->c.visc_const ? 1.0 : (ST + 1.0) * pow(s->T[n], 1.5) / (ST + s->T[n]);
  }
}

/* Modified Ducros sensor (shock_sensors.py:12-49, metric-transformed: d/dx0 = d/dxi0, d/dx1 =
 * D11 d/dxi1), evaluated on the interior with the one-sided closures of the derivatives:
 *   theta = (1/2 - 1/2 tanh(2.5 (1 + 100 div))) div^2 / (eps + div^2 + omega^2),
 *   div = du0/dx0 + du1/dx1, omega = du1/dx0 - du0/dx1. */
static void sensor(s2_t *s) {
  FOR2(0, N0, 0, N1) {
    const size_t n = I2(s, i, j);
    const double l0 = d1c(s, s->u0, i, j, 0), l1 = d1c(s, s->u1, i, j, 0);
    const double l2 = d1c(s, s->u0, i, j, 1), l3 = d1c(s, s->u1, i, j, 1);
    const double D = s->D11[n];
    const double div = l0 + l3 * D, om = l1 - l2 * D;
    s->theta[n] = (0.5 - 0.5 * tanh(250.0 * l0 + 250.0 * l3 * D + 2.5)) * (div * div) /
                  (s->c.sensor_eps + div * div + om * om);
  }
}

/* TENO cut-off at the interface whose left point is n: fixed, or from the sensor there */
static double teno_cutoff(const s2_t *s, size_t n) {
  if (!s->c.teno_adaptive) return s->c.teno_ct;
  const double th = s->theta[n];
  return pow(10.0, -floor(s->c.teno_a1 - s->c.teno_a2 * (-pow(1 - th, 4) * (4 * th + 1) + 1)));
}

/* ---------------------------------------------------------------------------------------------
 * TENO5 with fixed cut-off (schemes/spatial/teno.py:57-213, 407-465): smoothness indicators of the
 * half-split fluxes, alpha_r = (1 + |b0 - b2|/(eps + b_r))^6, delta_r = 0 if alpha_r/sum < C_T,
 * omega_r = d_r delta_r / sum(d delta), d = (11/20, 2/5, 1/20) for the central, downwind and
 * upwind candidates.  f = CF +- lambda CS at points i-2..i+2 (right-going side).
 * ------------------------------------------------------------------------------------------- */
static double teno5_plus(const s2_t *s, const double f[5], double CT) {
  const double eps = s->c.teno_eps;
  const double h0 = 0.5 * f[0], h1 = 0.5 * f[1], h2 = 0.5 * f[2], h3 = 0.5 * f[3], h4 = 0.5 * f[4];
  const double b0 = 0.25 * (h1 - h3) * (h1 - h3) + (13.0 / 12.0) * (h1 - 2 * h2 + h3) * (h1 - 2 * h2 + h3);
  const double b1 = (13.0 / 12.0) * (h2 - 2 * h3 + h4) * (h2 - 2 * h3 + h4) + 0.25 * (3 * h2 - 4 * h3 + h4) * (3 * h2 - 4 * h3 + h4);
  const double b2 = 0.25 * (h0 - 4 * h1 + 3 * h2) * (h0 - 4 * h1 + 3 * h2) + (13.0 / 12.0) * (h0 - 2 * h1 + h2) * (h0 - 2 * h1 + h2);
  const double tau = fabs(b0 - b2);
  const double a0 = pow(1 + tau / (eps + b0), 6), a1 = pow(1 + tau / (eps + b1), 6), a2 = pow(1 + tau / (eps + b2), 6);
  const double inv = 1.0 / (a0 + a1 + a2);
  const double d0 = CT > a0 * inv ? 0.0 : 1.0, d1 = CT > a1 * inv ? 0.0 : 1.0, d2 = CT > a2 * inv ? 0.0 : 1.0;
  const double iw = 1.0 / (0.55 * d0 + 0.4 * d1 + 0.05 * d2);
  return 0.55 * d0 * iw * (-(1.0 / 12.0) * f[1] + (5.0 / 12.0) * f[2] + (1.0 / 6.0) * f[3]) +
         0.4 * d1 * iw * ((1.0 / 6.0) * f[2] + (5.0 / 12.0) * f[3] - (1.0 / 12.0) * f[4]) +
         0.05 * d2 * iw * ((1.0 / 6.0) * f[0] - (7.0 / 12.0) * f[1] + (11.0 / 12.0) * f[2]);
}

/* Characteristic fluxes (TENO5, WENO5-JS, WENO5-Z or TENO6, as the configuration says) in direction
 * dir with Roe averaging and the 2D Euler eigensystem for a unit normal (physical_models/euler_eigensystem.py:77-105; the block's metric is diagonal, so the
 * eigensystem is Cartesian and the metric enters the residual only). */
static void teno_fluxes(s2_t *s, int dir) {
  const double g = s->c.gama;
  const int lo0 = dir == 0 ? -1 : 0, lo1 = dir == 1 ? -1 : 0;
  const size_t o = dir == 0 ? 1 : (size_t)s->px;
  const int e = 1 - dir;                   /* the other axis */
  const double sg = dir == 0 ? 1.0 : -1.0; /* sign of the shear row */
  FOR2(lo0, N0, lo1, N1) {
    const size_t c = I2(s, i, j);
    const double rl = s->q[0][c], rr = s->q[0][c + o];
    const double uL[2] = {s->u0[c], s->u1[c]}, uR[2] = {s->u0[c + o], s->u1[c + o]};
    double u[2], rho, a;
    if (s->c.simple_avg) { /* SimpleAverage (averaging.py:31-59) */
      rho = 0.5 * (rl + rr);
      for (int k = 0; k < 2; ++k) u[k] = 0.5 * (uL[k] + uR[k]);
      a = 0.5 * (s->a[c] + s->a[c + o]);
    } else { /* RoeAverage (averaging.py:62-114) */
      const double sl = sqrt(rl), sr = sqrt(rr), inv = 1.0 / (sl + sr);
      rho = sqrt(rl * rr);
      for (int k = 0; k < 2; ++k) u[k] = inv * (sl * uL[k] + sr * uR[k]);
      const double Hh = inv * ((s->p[c] + s->q[3][c]) / sl + (s->p[c + o] + s->q[3][c + o]) / sr);
      a = sqrt((g - 1) * (Hh - 0.5 * (u[0] * u[0] + u[1] * u[1])));
    }
    const double phi = (g - 1) * 0.5 * (u[0] * u[0] + u[1] * u[1]);
    const double bt = 1.0 / (rho * a * sqrt(2.0)), al = rho / (a * sqrt(2.0));
    double L[4][4];
    /* row 0: entropy; row 1: shear; rows 2, 3: u_d + a, u_d - a */
    L[0][0] = 1 - phi / (a * a);
    L[0][1] = (g - 1) * u[0] / (a * a);
    L[0][2] = (g - 1) * u[1] / (a * a);
    L[0][3] = -(g - 1) / (a * a);
    L[1][0] = sg * u[e] / rho;
    L[1][1 + dir] = 0.0;
    L[1][1 + e] = -sg / rho;
    L[1][3] = 0.0;
    for (int w = 0; w < 2; ++w) {
      const double sgn = w == 0 ? 1.0 : -1.0;
      L[2 + w][0] = bt * (phi - sgn * a * u[dir]);
      for (int k = 0; k < 2; ++k) L[2 + w][1 + k] = -bt * ((g - 1) * u[k] - (k == dir ? sgn * a : 0.0));
      L[2 + w][3] = bt * (g - 1);
    }
    double CF[4][6], CS[4][6], lam[4] = {0, 0, 0, 0};
    for (int t = 0; t < 6; ++t) {
      const size_t m = c + (size_t)((long)(t - 2) * (long)o);
      const double un = dir == 0 ? s->u0[m] : s->u1[m];
      double Fv[4], Q[4];
      for (int v = 0; v < 4; ++v) Q[v] = s->q[v][m];
      Fv[0] = s->q[1 + dir][m];
      for (int k = 0; k < 2; ++k) Fv[1 + k] = s->q[1 + k][m] * un + (k == dir ? s->p[m] : 0.0);
      Fv[3] = (s->p[m] + s->q[3][m]) * un;
      for (int r = 0; r < 4; ++r) {
        double cf = 0, cs = 0;
        for (int v = 0; v < 4; ++v) { cf += L[r][v] * Fv[v]; cs += L[r][v] * Q[v]; }
        CF[r][t] = cf;
        CS[r][t] = cs;
      }
      const double ev[4] = {fabs(un), fabs(un), fabs(un + s->a[m]), fabs(s->a[m] - un)};
      for (int r = 0; r < 4; ++r) lam[r] = fmax(lam[r], ev[r]);
    }
    double rec[4];
    const double CT = teno_cutoff(s, c);
    const int conv = s->c.conv;
    for (int r = 0; r < 4; ++r) {
      double fp[5], fm[5];
      for (int t = 0; t < 5; ++t) {
        fp[t] = CF[r][t] + lam[r] * CS[r][t];
        fm[t] = CF[r][5 - t] - lam[r] * CS[r][5 - t];
      }
      if (conv == OSBO_CONV_WENO5JS || conv == OSBO_CONV_WENO5Z) {
        /* weno.py:341-369 (JS) and 283-331 (Z): + side on points i-2..i+2, - side on i-1..i+3 */
        double g[5];
        for (int t = 0; t < 5; ++t) g[t] = CF[r][t + 1] - lam[r] * CS[r][t + 1];
        const int z = conv == OSBO_CONV_WENO5Z;
        rec[r] = osbo_side_weno5_plus(fp, z) + osbo_side_weno5_minus(g, z);
      } else if (conv == OSBO_CONV_TENO6) {
        /* teno.py:94-192, 216-234: both sides on the six points */
        double gp[6], gm[6];
        for (int t = 0; t < 6; ++t) {
          gp[t] = CF[r][t] + lam[r] * CS[r][t];
          gm[t] = CF[r][t] - lam[r] * CS[r][t];
        }
        rec[r] = osbo_side_teno6(gp, 1, s->c.teno_eps, CT) + osbo_side_teno6(gm, 0, s->c.teno_eps, CT);
      } else {
        rec[r] = teno5_plus(s, fp, CT) + teno5_plus(s, fm, CT);
      }
    }
    /* REV columns (euler_eigensystem.py:90-92) */
    const double hh = (phi + a * a) / (g - 1);
    double out[4];
    out[0] = rec[0] + al * (rec[2] + rec[3]);
    for (int k = 0; k < 2; ++k)
      out[1 + k] = u[k] * rec[0] + al * (u[k] * (rec[2] + rec[3]) + (k == dir ? a * (rec[2] - rec[3]) : 0.0));
    out[3] = (phi / (g - 1)) * rec[0] + al * (hh * (rec[2] + rec[3]) + u[dir] * a * (rec[2] - rec[3]));
    out[1 + e] += -sg * rho * rec[1];
    out[3] += -sg * rho * u[e] * rec[1];
    for (int v = 0; v < 4; ++v) s->flux[v][c] = out[v];
  }
}

/* LLFTeno residual (shock_capturing.py:21-34, opensblifunctions.py:658-676): x0 uniform, x1 through
 * D11: R = -(F_i - F_{i-1})/delta0 - D11 (G_j - G_{j-1})/delta1 */
static void residual_teno(s2_t *s) {
  teno_fluxes(s, 0);
  FOR2(0, N0, 0, N1) {
    const size_t c = I2(s, i, j);
    for (int v = 0; v < 4; ++v) s->res[v][c] = -(s->flux[v][c] - s->flux[v][c - 1]) / s->c.delta[0];
  }
  teno_fluxes(s, 1);
  FOR2(0, N0, 0, N1) {
    const size_t c = I2(s, i, j);
    for (int v = 0; v < 4; ++v)
      s->res[v][c] -= (s->flux[v][c] - s->flux[v][c - s->px]) / s->c.delta[1] * s->D11[c];
  }
}

/* Central skew-symmetric convective terms (laminar_channel.py's Skew(...); the same form as the
 * Taylor-Green script, parsing.py:75-111) on a Cartesian block with the derivative closures of the
 * faces, and the forcing c_j:
 *   R_rho = -sum_j skew(rho, j), R_rhou_i = -sum_j skew(rhou_i, j) - dp/dx_i - c_i,
 *   R_rhoE = -sum_j skew(rhoE, j) - sum_j d(p u_j)/dx_j - c_j u_j,
 *   skew(phi, j) = (d(phi u_j)/dx_j + u_j dphi/dx_j + phi du_j/dx_j) / 2. */
static void residual_skew(s2_t *s) {
  double *prod = alloc2(s);
  const double *U[2] = {s->u0, s->u1};
  const double *phi[4] = {s->q[0], s->q[1], s->q[2], s->q[3]};
  for (int v = 0; v < 4; ++v) FOR2(0, N0, 0, N1) s->res[v][I2(s, i, j)] = 0.0;
  for (int v = 0; v < 4; ++v)
    for (int d = 0; d < 2; ++d) {
      FOR2(-H, N0 + H, -H, N1 + H) prod[I2(s, i, j)] = phi[v][I2(s, i, j)] * U[d][I2(s, i, j)];
      FOR2(0, N0, 0, N1) {
        const size_t c = I2(s, i, j);
        const double sk = 0.5 * (d1c(s, prod, i, j, d) + U[d][c] * d1c(s, phi[v], i, j, d) + phi[v][c] * d1c(s, U[d], i, j, d));
        s->res[v][c] -= sk;
      }
    }
  for (int d = 0; d < 2; ++d) {
    FOR2(0, N0, 0, N1) s->res[1 + d][I2(s, i, j)] -= d1c(s, s->p, i, j, d);
    FOR2(-H, N0 + H, -H, N1 + H) prod[I2(s, i, j)] = s->p[I2(s, i, j)] * U[d][I2(s, i, j)];
    FOR2(0, N0, 0, N1) s->res[3][I2(s, i, j)] -= d1c(s, prod, i, j, d);
  }
  FOR2(0, N0, 0, N1) {
    const size_t c = I2(s, i, j);
    s->res[1][c] -= s->c.force[0];
    s->res[2][c] -= s->c.force[1];
    s->res[3][c] -= s->c.force[0] * s->u0[c] + s->c.force[1] * s->u1[c];
  }
  free(prod);
}

/* Viscous and heat-flux terms with Sutherland viscosity in the stretched metric
 * (katzer_SBLI.py:12-14; metric.py:72-234): d/dx0 = d/dxi0, d/dx1 = D11 d/dxi1,
 * d2/dx1^2 = D11^2 d2/dxi1^2 + D11 SD111 d/dxi1, d2/dx0dx1 = D11 d/dxi1 (d/dxi0) (inner derivative
 * over the extended xi1 range); every derivative uses the one-sided closures at the boundaries.
 *   mom_i += d_j tau_ij, tau_ij = mu/Re (d_j u_i + d_i u_j - 2/3 delta_ij div u)
 *   energy += d_j (u_i tau_ij) + d_j (kappa mu d_j T), kappa = 1/((gama-1) Minf^2 Pr Re) */
static void residual_viscous(s2_t *s) {
  const double Re = s->c.Re;
  const double kap = 1.0 / ((s->c.gama - 1) * s->c.Minf * s->c.Minf * s->c.Pr * Re);
  double *du0x = alloc2(s), *du1x = alloc2(s);
  FOR2(0, N0, -2, N1 + 2) {
    du0x[I2(s, i, j)] = d1c(s, s->u0, i, j, 0);
    du1x[I2(s, i, j)] = d1c(s, s->u1, i, j, 0);
  }
  FOR2(0, N0, 0, N1) {
    const size_t c = I2(s, i, j);
    const double D = s->D11[c], S = s->SD111[c], mu = s->mu[c];
    const double u[2] = {s->u0[c], s->u1[c]};
    double g[2][2], h[2][2][2];
    g[0][0] = du0x[c];
    g[1][0] = du1x[c];
    g[0][1] = D * d1c(s, s->u0, i, j, 1);
    g[1][1] = D * d1c(s, s->u1, i, j, 1);
    const double mux = d1c(s, s->mu, i, j, 0), muy = D * d1c(s, s->mu, i, j, 1);
    const double Tx = d1c(s, s->T, i, j, 0), Ty = D * d1c(s, s->T, i, j, 1);
    const double Txx = d2c(s, s->T, i, j, 0), Tyy = D * D * d2c(s, s->T, i, j, 1) + D * S * d1c(s, s->T, i, j, 1);
    const double *uc[2] = {s->u0, s->u1};
    const double *dux[2] = {du0x, du1x};
    for (int k = 0; k < 2; ++k) {
      h[k][0][0] = d2c(s, uc[k], i, j, 0);
      h[k][1][1] = D * D * d2c(s, uc[k], i, j, 1) + D * S * d1c(s, uc[k], i, j, 1);
      h[k][0][1] = h[k][1][0] = D * d1c(s, dux[k], i, j, 1);
    }
    const double div = g[0][0] + g[1][1];
    double tau[2][2], dtau[2];
    const double mug[2] = {mux, muy};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) tau[a][b] = mu / Re * (g[a][b] + g[b][a] - (a == b ? 2.0 / 3.0 * div : 0.0));
    for (int a = 0; a < 2; ++a) {
      /* d_b tau_ab = (1/Re)[ mu_b (..) + mu (lap u_a + d_a div u - 2/3 d_a div u) ] */
      double v = 0.0;
      for (int b = 0; b < 2; ++b) v += mug[b] * (g[a][b] + g[b][a] - (a == b ? 2.0 / 3.0 * div : 0.0)) / Re;
      const double lap = h[a][0][0] + h[a][1][1];
      const double ddiv = h[0][a][0] + h[1][a][1];
      v += mu / Re * (lap + ddiv / 3.0);
      dtau[a] = v;
      s->res[1 + a][c] += v;
    }
    double e = kap * (mu * (Txx + Tyy) + mux * Tx + muy * Ty);
    for (int a = 0; a < 2; ++a) {
      for (int b = 0; b < 2; ++b) e += tau[a][b] * g[a][b];
      e += u[a] * dtau[a];
    }
    s->res[3][c] += e;
  }
  free(du0x);
  free(du1x);
}

int osbo2d_run(const osbo2d_cfg *cfg, double *q, int nsteps) {
  s2_t s;
  s2_init(&s, cfg);
  const int hp = 4, pxo = cfg->n[0] + 2 * hp, pyo = cfg->n[1] + 2 * hp;
  for (int v = 0; v < 4; ++v)
    for (int j = -hp; j < cfg->n[1] + hp; ++j)
      for (int i = -hp; i < cfg->n[0] + hp; ++i)
        s.q[v][I2(&s, i, j)] = q[((size_t)v * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)];
  metrics(&s);
  for (int it = 0; it < nsteps; ++it) {
    apply_bcs(&s);
    if (cfg->rk2reg) /* "Save equations": qold = q (the RK register du holds qold) */
      for (int v = 0; v < 4; ++v)
        for (int j = 0; j < cfg->n[1]; ++j)
          for (int i = 0; i < cfg->n[0]; ++i) s.du[v][I2(&s, i, j)] = s.q[v][I2(&s, i, j)];
    for (int st = 0; st < 3; ++st) {
      constituent(&s);
      if (cfg->teno_adaptive) sensor(&s);
      if (cfg->skew) residual_skew(&s);
      else residual_teno(&s);
      if (!cfg->euler) residual_viscous(&s);
      for (int v = 0; v < 4; ++v)
        for (int j = 0; j < cfg->n[1]; ++j)
          for (int i = 0; i < cfg->n[0]; ++i) {
            const size_t c = I2(&s, i, j);
            if (cfg->rk2reg) { /* rk_sbli.py:117-124: sub stage, then the temporal register */
              s.q[v][c] = cfg->dt * cfg->rkB[st] * s.res[v][c] + s.du[v][c];
              s.du[v][c] = cfg->dt * cfg->rkA[st] * s.res[v][c] + s.du[v][c];
            } else { /* RungeKuttaLS (rk_LS.py:155-166): du = A du + dt R; q = q + B du */
              s.du[v][c] = cfg->dt * s.res[v][c] + cfg->rkA[st] * s.du[v][c];
              s.q[v][c] = cfg->rkB[st] * s.du[v][c] + s.q[v][c];
            }
          }
      apply_bcs(&s);
    }
  }
  for (int v = 0; v < 4; ++v)
    for (int j = -hp; j < cfg->n[1] + hp; ++j)
      for (int i = -hp; i < cfg->n[0] + hp; ++i)
        q[((size_t)v * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)] = s.q[v][I2(&s, i, j)];
  s2_free(&s);
  return 0;
}

/* The right-hand side of a padded state (boundary conditions applied first) on the interior,
 * [4][n1][n0]. */
int osbo2d_residual(const osbo2d_cfg *cfg, const double *q, double *r) {
  s2_t s;
  s2_init(&s, cfg);
  const int hp = 4, pxo = cfg->n[0] + 2 * hp, pyo = cfg->n[1] + 2 * hp;
  for (int v = 0; v < 4; ++v)
    for (int j = -hp; j < cfg->n[1] + hp; ++j)
      for (int i = -hp; i < cfg->n[0] + hp; ++i)
        s.q[v][I2(&s, i, j)] = q[((size_t)v * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)];
  metrics(&s);
  apply_bcs(&s);
  constituent(&s);
  if (cfg->teno_adaptive) sensor(&s);
  if (cfg->skew) residual_skew(&s);
  else residual_teno(&s);
  if (!cfg->euler) residual_viscous(&s);
  size_t m = 0;
  for (int v = 0; v < 4; ++v)
    for (int j = 0; j < cfg->n[1]; ++j)
      for (int i = 0; i < cfg->n[0]; ++i) r[m++] = s.res[v][I2(&s, i, j)];
  s2_free(&s);
  return 0;
}

/* The adaptive TENO cut-off of a padded state (the boundary conditions applied first) over the
 * interior, [n1][n0]: the field the reference stores as TENO_B0. */
int osbo2d_cutoff(const osbo2d_cfg *cfg, const double *q, double *ct) {
  s2_t s;
  s2_init(&s, cfg);
  const int hp = 4, pxo = cfg->n[0] + 2 * hp, pyo = cfg->n[1] + 2 * hp;
  for (int v = 0; v < 4; ++v)
    for (int j = -hp; j < cfg->n[1] + hp; ++j)
      for (int i = -hp; i < cfg->n[0] + hp; ++i)
        s.q[v][I2(&s, i, j)] = q[((size_t)v * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)];
  metrics(&s);
  apply_bcs(&s);
  constituent(&s);
  sensor(&s);
  for (int j = 0; j < cfg->n[1]; ++j)
    for (int i = 0; i < cfg->n[0]; ++i) ct[(size_t)j * cfg->n[0] + i] = teno_cutoff(&s, I2(&s, i, j));
  s2_free(&s);
  return 0;
}

int osbo2d_metrics(const osbo2d_cfg *cfg, double *D11, double *SD111) {
  s2_t s;
  s2_init(&s, cfg);
  metrics(&s);
  for (int j = 0; j < cfg->n[1]; ++j)
    for (int i = 0; i < cfg->n[0]; ++i) {
      D11[(size_t)j * cfg->n[0] + i] = s.D11[I2(&s, i, j)];
      SD111[(size_t)j * cfg->n[0] + i] = s.SD111[I2(&s, i, j)];
    }
  s2_free(&s);
  return 0;
}
