/* osb_oracle3w.c -- CPU restatement (FP64) of the generated per-timestep algorithm for a 3D
 * span-periodic wall-bounded block: the 2D shock/boundary-layer configuration of osb_oracle2d.c with
 * a periodic x2 axis (apps/transitional_SBLI/transitional_SBLI.py without its statistics and
 * restart), and the channel configuration (apps/channel_flow/compressible_TCF_TENO/
 * turbulent_channel.py without its statistics): periodic x0, isothermal walls on both x1 faces,
 * mu = T^0.7 and the constant forcing of the momentum and energy equations.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle).  See osb_oracle.h.
 *
 * Kernel order (algorithm.py:384-477):
 *   before the loop: coordinates, metric derivative, D11 = 1/(dx1/dxi1), metric halos, SD111
 *   iter { BCs; stage { CRs; fluxes x0, x1, x2; flux residual; viscous terms; LS-RK update; BCs } }
 *   BCs = inlet (x0 side 0), outlet (x0 side 1), isothermal wall (x1 side 0), Dirichlet (x1 side 1),
 *         then the periodic exchange of x2 (exchange.py:9-57);
 *   channel: the periodic exchange of x0, isothermal walls on both x1 faces, the exchange of x2.
 * The faces are pointwise in x2, so applying them to the interior planes and then wrapping the x2
 * halos gives what the generated code gives by applying them over the x2 halo range as well; the
 * wall faces are pointwise in x0 too, so wrapping x0 after them equals wrapping it before.
 * Arrays carry a 5-point halo; the state exchanged with callers carries a 4-point halo.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "osb_oracle.h"

#define H 5

/* reconstruction sides and eigensystem of the 3D restatement (osb_oracle.c), Carpenter weights of
 * the 2D one (osb_oracle2d.c) */
double osbo_side_weno5_plus(const double f[5], int z);
double osbo_side_weno5_minus(const double g[5], int z);
double osbo_side_teno6(const double g[6], int plus, double eps, double CT);
double osbo_side_teno5(const double f[5], double eps, double CT);
void osbo_eigensystem3(int dir, double rho, double u0, double u1, double u2, double a, double g, double L[5][5],
                       double R[5][5]);
void osbo2d_carpenter_d1(double *c24);

typedef struct {
  osbo3w_cfg c;
  int px, py, pz;
  size_t np;
  double *q[5], *du[5], *res[5], *flux[5];
  double *u[3], *p, *a, *T, *mu;
  double *wk[3];                 /* inner x0 derivatives of u_i (nested derivatives) */
  double *theta;                 /* Ducros sensor (adaptive TENO), interior; 0 elsewhere */
  double *wz[3];                 /* inner x2 derivatives of u_i */
  double x1[256 + 2 * H], D11[256 + 2 * H], SD111[256 + 2 * H]; /* functions of x1 only */
  double carp[4][6];
} s3_t;

static inline size_t I3(const s3_t *s, int i, int j, int k) {
  return (size_t)(i + H) + (size_t)s->px * ((size_t)(j + H) + (size_t)s->py * (size_t)(k + H));
}
static double *alloc3(const s3_t *s) { return (double *)calloc(s->np, sizeof(double)); }

#define N0 (s->c.n[0])
#define N1 (s->c.n[1])
#define N2 (s->c.n[2])
#define FOR3(i0, i1, j0, j1, k0, k1)  \
  for (int k = (k0); k < (k1); ++k)   \
    for (int j = (j0); j < (j1); ++j) \
      for (int i = (i0); i < (i1); ++i)

static int s3_init(s3_t *s, const osbo3w_cfg *cfg) {
  memset(s, 0, sizeof(*s));
  s->c = *cfg;
  if (cfg->n[1] > 256 || cfg->n[2] < 4 || (cfg->periodic0 && cfg->n[0] < H)) return -1;
  double c24[24];
  osbo2d_carpenter_d1(c24);
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) s->carp[r][m] = c24[6 * r + m];
  s->px = cfg->n[0] + 2 * H;
  s->py = cfg->n[1] + 2 * H;
  s->pz = cfg->n[2] + 2 * H;
  s->np = (size_t)s->px * s->py * s->pz;
  for (int v = 0; v < 5; ++v) {
    s->q[v] = alloc3(s);
    s->du[v] = alloc3(s);
    s->res[v] = alloc3(s);
    s->flux[v] = alloc3(s);
  }
  for (int d = 0; d < 3; ++d) {
    s->u[d] = alloc3(s);
    s->wk[d] = alloc3(s);
    s->wz[d] = alloc3(s);
  }
  s->p = alloc3(s);
  s->theta = alloc3(s);
  s->a = alloc3(s);
  s->T = alloc3(s);
  s->mu = alloc3(s);
  return 0;
}

static void s3_free(s3_t *s) {
  for (int v = 0; v < 5; ++v) {
    free(s->q[v]);
    free(s->du[v]);
    free(s->res[v]);
    free(s->flux[v]);
  }
  for (int d = 0; d < 3; ++d) {
    free(s->u[d]);
    free(s->wk[d]);
    free(s->wz[d]);
  }
  free(s->p);
  free(s->theta);
  free(s->a);
  free(s->T);
  free(s->mu);
}

/* ---------------------------------------------------------------------------------------------
 * 4th-order central derivatives with the one-sided closures of the x0 and x1 faces (as in
 * osb_oracle2d.c: ReducedAccess, reduced_access_scheme.py:34-83, or Carpenter,
 * Carpenter_scheme.py:6-102); x2 is periodic, every point takes the central stencil.
 * ------------------------------------------------------------------------------------------- */
static int periodic_axis(const s3_t *s, int dir) { return dir == 2 || (dir == 0 && s->c.periodic0); }

static double d1_stencil(const s3_t *s, int dir, int kk, int n, double (*G)(const void *, int), const void *ctx) {
  if (periodic_axis(s, dir))
    return (1.0 / 12.0) * G(ctx, -2) - (2.0 / 3.0) * G(ctx, -1) + (2.0 / 3.0) * G(ctx, 1) - (1.0 / 12.0) * G(ctx, 2);
  const int c0 = s->c.closure[dir][0], c1 = s->c.closure[dir][1];
  int side = -1, r = 0;
  if (kk < (c0 == 1 ? 4 : 2)) side = 0, r = kk;
  else if (n - 1 - kk < (c1 == 1 ? 4 : 2)) side = 1, r = n - 1 - kk;
  const int carp = side >= 0 && (side == 0 ? c0 : c1) == 1;
  double v;
  if (carp) {
    v = 0.0;
    for (int m = 0; m < 6; ++m) v += s->carp[r][m] * (side == 0 ? G(ctx, m - r) : G(ctx, r - m));
    if (side == 1) v = -v;
  } else if (side == 0 && r == 0)
    v = -(25.0 / 12.0) * G(ctx, 0) + 4.0 * G(ctx, 1) - 3.0 * G(ctx, 2) + (4.0 / 3.0) * G(ctx, 3) - 0.25 * G(ctx, 4);
  else if (side == 0)
    v = -0.25 * G(ctx, -1) - (5.0 / 6.0) * G(ctx, 0) + 1.5 * G(ctx, 1) - 0.5 * G(ctx, 2) + (1.0 / 12.0) * G(ctx, 3);
  else if (side == 1 && r == 0)
    v = (25.0 / 12.0) * G(ctx, 0) - 4.0 * G(ctx, -1) + 3.0 * G(ctx, -2) - (4.0 / 3.0) * G(ctx, -3) + 0.25 * G(ctx, -4);
  else if (side == 1)
    v = 0.25 * G(ctx, 1) + (5.0 / 6.0) * G(ctx, 0) - 1.5 * G(ctx, -1) + 0.5 * G(ctx, -2) - (1.0 / 12.0) * G(ctx, -3);
  else
    v = (1.0 / 12.0) * G(ctx, -2) - (2.0 / 3.0) * G(ctx, -1) + (2.0 / 3.0) * G(ctx, 1) - (1.0 / 12.0) * G(ctx, 2);
  return v;
}

static double d2_stencil(const s3_t *s, int dir, int kk, int n, double (*G)(const void *, int), const void *ctx) {
  if (periodic_axis(s, dir))
    return -(1.0 / 12.0) * G(ctx, -2) + (4.0 / 3.0) * G(ctx, -1) - 2.5 * G(ctx, 0) + (4.0 / 3.0) * G(ctx, 1) -
           (1.0 / 12.0) * G(ctx, 2);
  if (kk == 0)
    return (35.0 / 12.0) * G(ctx, 0) - (26.0 / 3.0) * G(ctx, 1) + 9.5 * G(ctx, 2) - (14.0 / 3.0) * G(ctx, 3) +
           (11.0 / 12.0) * G(ctx, 4);
  if (kk == 1)
    return (11.0 / 12.0) * G(ctx, -1) - (5.0 / 3.0) * G(ctx, 0) + 0.5 * G(ctx, 1) + (1.0 / 3.0) * G(ctx, 2) -
           (1.0 / 12.0) * G(ctx, 3);
  if (kk == n - 1)
    return (35.0 / 12.0) * G(ctx, 0) - (26.0 / 3.0) * G(ctx, -1) + 9.5 * G(ctx, -2) - (14.0 / 3.0) * G(ctx, -3) +
           (11.0 / 12.0) * G(ctx, -4);
  if (kk == n - 2)
    return (11.0 / 12.0) * G(ctx, 1) - (5.0 / 3.0) * G(ctx, 0) + 0.5 * G(ctx, -1) + (1.0 / 3.0) * G(ctx, -2) -
           (1.0 / 12.0) * G(ctx, -3);
  return -(1.0 / 12.0) * G(ctx, -2) + (4.0 / 3.0) * G(ctx, -1) - 2.5 * G(ctx, 0) + (4.0 / 3.0) * G(ctx, 1) -
         (1.0 / 12.0) * G(ctx, 2);
}

typedef struct {
  const s3_t *s;
  const double *f;
  int i, j, k, dir;
} pt_t;

static double G3(const void *ctx, int o) {
  const pt_t *p = (const pt_t *)ctx;
  int i = p->i, j = p->j, k = p->k;
  if (p->dir == 0) i += o;
  else if (p->dir == 1) j += o;
  else k += o;
  return p->f[I3(p->s, i, j, k)];
}

static double d1c(const s3_t *s, const double *f, int i, int j, int k, int dir) {
  const pt_t p = {s, f, i, j, k, dir};
  const int n = dir == 0 ? N0 : dir == 1 ? N1 : N2, kk = dir == 0 ? i : dir == 1 ? j : k;
  return (1.0 / s->c.delta[dir]) * d1_stencil(s, dir, kk, n, G3, &p);
}

static double d2c(const s3_t *s, const double *f, int i, int j, int k, int dir) {
  const pt_t p = {s, f, i, j, k, dir};
  const int n = dir == 0 ? N0 : dir == 1 ? N1 : N2, kk = dir == 0 ? i : dir == 1 ? j : k;
  return (1.0 / (s->c.delta[dir] * s->c.delta[dir])) * d2_stencil(s, dir, kk, n, G3, &p);
}

/* ---------------------------------------------------------------------------------------------
 * Metrics (equation_types/metric.py:37-234, 315-332), stretched in x1 only, so functions of j:
 * x1(j) = Lx1 sinh(by delta1 j / Lx1) / sinh(by) (or the channel's tanh clustering), D11 =
 * 1/(dx1/dxi1) with the x1 closures, halos mirrored about the boundary points, SD111 = dD11/dxi1.
 * ------------------------------------------------------------------------------------------- */
static double G1(const void *ctx, int o) { return ((const double *)ctx)[o]; }

static void metrics(s3_t *s) {
  const double Lx1 = s->c.Lx1, by = s->c.by, d1 = s->c.delta[1];
  for (int j = -3; j < N1 + 4; ++j)
    s->x1[j + H] = s->c.grid_tanh /* turbulent_channel.py:167-170, Ly = 2 */
                       ? 0.5 * 2.0 * (1.0 - tanh(s->c.stretch * (1.0 - 2.0 * (j / (N1 - 1.0)))) / tanh(s->c.stretch)) - 1.0
                       : sinh(d1 * by * (1.0 / Lx1) * j) / ((1.0 / Lx1) * sinh(by));
  double wk[256 + 2 * H];
  for (int j = 0; j < N1; ++j) wk[j + H] = (1.0 / d1) * d1_stencil(s, 1, j, N1, G1, &s->x1[j + H]);
  for (int j = 0; j < N1; ++j) s->D11[j + H] = 1.0 / wk[j + H];
  for (int t = 1; t <= 3; ++t) s->D11[-t + H] = s->D11[t + H];
  for (int t = 1; t <= 4; ++t) s->D11[N1 - 1 + t + H] = s->D11[N1 - 1 - t + H];
  for (int j = 0; j < N1; ++j) s->SD111[j + H] = (1.0 / d1) * d1_stencil(s, 1, j, N1, G1, &s->D11[j + H]);
}

/* ---------------------------------------------------------------------------------------------
 * Boundary conditions (as osb_oracle2d.c, with the spanwise momentum): inlet, outlet, wall, top
 * on every interior x2 plane, then the x2 wrap of every halo plane.
 * ------------------------------------------------------------------------------------------- */
static void apply_bcs(s3_t *s) {
  const double g = s->c.gama, M = s->c.Minf, Tw = s->c.Twall;
  for (int k = 0; k < N2; ++k) {
    for (int j = -3; j < N1 + 4 && !s->c.periodic0; ++j) { /* InletPressureExtrapolateBC (inlet_pressure_extrapolate.py:11-66) */
      const size_t b = I3(s, 0, j, k);
      const double rhob = s->q[0][b];
      const double ub0 = fabs(s->q[1][b] / rhob), ub1 = fabs(s->q[2][b] / rhob), ub2 = fabs(s->q[3][b] / rhob);
      const double pb = (g - 1) * (-0.5 * rhob * (ub0 * ub0 + ub1 * ub1 + ub2 * ub2) + s->q[4][b]);
      const double ab = sqrt(g * pb / rhob);
      if (ub0 >= ab) {
        for (int v = 0; v < 5; ++v) s->q[v][b] = s->q[v][I3(s, -1, j, k)];
      } else {
        for (int t = 1; t <= 3; ++t) s->q[4][I3(s, -t, j, k)] = s->q[4][b];
      }
    }
    for (int j = -3; j < N1 + 4 && !s->c.periodic0; ++j) /* ExtrapolationBC order 0 (extrapolation.py:8-58) */
      for (int v = 0; v < 5; ++v) {
        const double val = s->q[v][I3(s, N0 - 2, j, k)];
        for (int t = 0; t <= 4; ++t) s->q[v][I3(s, N0 - 1 + t, j, k)] = val;
      }
    for (int i = -3; i < N0 + 4; ++i) { /* IsothermalWallBC (isothermal_wall.py:32-88) */
      const size_t w = I3(s, i, 0, k), a1 = I3(s, i, 1, k);
      s->q[1][w] = 0.0;
      s->q[2][w] = 0.0;
      s->q[3][w] = 0.0;
      s->q[4][w] = Tw * (1.0 / (M * M)) * s->q[0][w] / (g * (g - 1.0));
      const double Pw = (g - 1) * (-(0.5 * s->q[1][w] * s->q[1][w] + 0.5 * s->q[2][w] * s->q[2][w] +
                                     0.5 * s->q[3][w] * s->q[3][w]) / s->q[0][w] + s->q[4][w]);
      const double Ta = M * M * g * (g - 1) *
                        (-(0.5 * s->q[1][a1] * s->q[1][a1] + 0.5 * s->q[2][a1] * s->q[2][a1] +
                           0.5 * s->q[3][a1] * s->q[3][a1]) / s->q[0][a1] + s->q[4][a1]) /
                        s->q[0][a1];
      for (int t = 1; t <= 3; ++t) {
        const size_t m = I3(s, i, t, k), h = I3(s, i, -t, k);
        const double um[3] = {s->q[1][m] / s->q[0][m], s->q[2][m] / s->q[0][m], s->q[3][m] / s->q[0][m]};
        const double Tt = (t + 1) * Tw - t * Ta;
        const double rh = M * M * g * Pw / Tt;
        s->q[0][h] = rh;
        for (int c = 0; c < 3; ++c) s->q[1 + c][h] = -rh * um[c];
        s->q[4][h] = (1.0 / (g - 1)) * Pw + 0.5 * rh * (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
      }
    }
    for (int i = -3; i < N0 + 4 && s->c.wall1; ++i) { /* IsothermalWallBC on side 1 (isothermal_wall.py:32-88) */
      const int jw = N1 - 1;
      const size_t w = I3(s, i, jw, k), a1 = I3(s, i, jw - 1, k);
      for (int c = 1; c <= 3; ++c) s->q[c][w] = 0.0;
      s->q[4][w] = Tw * (1.0 / (M * M)) * s->q[0][w] / (g * (g - 1.0));
      const double Pw = (g - 1) * s->q[4][w];
      const double Ta = M * M * g * (g - 1) *
                        (-(0.5 * s->q[1][a1] * s->q[1][a1] + 0.5 * s->q[2][a1] * s->q[2][a1] +
                           0.5 * s->q[3][a1] * s->q[3][a1]) / s->q[0][a1] + s->q[4][a1]) /
                        s->q[0][a1];
      for (int t = 1; t <= 4; ++t) {
        const size_t m = I3(s, i, jw - t, k), h = I3(s, i, jw + t, k);
        const double um[3] = {s->q[1][m] / s->q[0][m], s->q[2][m] / s->q[0][m], s->q[3][m] / s->q[0][m]};
        const double Tt = (t + 1) * Tw - t * Ta;
        const double rh = M * M * g * Pw / Tt;
        s->q[0][h] = rh;
        for (int c = 0; c < 3; ++c) s->q[1 + c][h] = -rh * um[c];
        s->q[4][h] = (1.0 / (g - 1)) * Pw + 0.5 * rh * (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
      }
    }
    for (int j = N1 - 1; j < N1 + 4 && !s->c.wall1; ++j) /* DirichletBC, piecewise in x0 */
      for (int i = -3; i < N0 + 4; ++i) {
        const double x0 = s->c.delta[0] * i;
        const double *st = s->c.dirichlet[x0 > s->c.x_switch ? 1 : 0];
        const size_t m = I3(s, i, j, k);
        if (s->c.dirichlet_ke) { /* rhou2 kept; rhoE from the face's rho and the local rhou2 */
          for (int v = 0; v < 3; ++v) s->q[v][m] = st[v];
          s->q[4][m] = st[4] + 0.5 * s->q[3][m] * s->q[3][m] / s->q[0][m];
        } else {
          for (int v = 0; v < 5; ++v) s->q[v][m] = st[v];
        }
      }
  }
  if (s->c.periodic0) /* periodic x0 */
    for (int v = 0; v < 5; ++v)
      for (int k = 0; k < N2; ++k)
        for (int j = -H; j < N1 + H; ++j)
          for (int i = -H; i < 0; ++i) {
            s->q[v][I3(s, i, j, k)] = s->q[v][I3(s, i + N0, j, k)];
            s->q[v][I3(s, N0 - 1 - i, j, k)] = s->q[v][I3(s, -1 - i, j, k)];
          }
  for (int v = 0; v < 5; ++v) /* periodic x2 */
    for (int k = -H; k < 0; ++k)
      for (int j = -H; j < N1 + H; ++j)
        for (int i = -H; i < N0 + H; ++i) {
          s->q[v][I3(s, i, j, k)] = s->q[v][I3(s, i, j, k + N2)];
          s->q[v][I3(s, i, j, N2 - 1 - k)] = s->q[v][I3(s, i, j, -1 - k)];
        }
}

/* Constituent relations (transitional_SBLI.py:33-38): u_i, p, a over -3..n+4 in x0, x1 and the x2
 * halos; T and mu (Sutherland, or the power law) over -2..n+2. */
static void constituent(s3_t *s) {
  const double g = s->c.gama, M = s->c.Minf, ST = s->c.SuthT / s->c.RefT;
  FOR3(-3, N0 + 4, -3, N1 + 4, -3, N2 + 3) {
    const size_t n = I3(s, i, j, k);
    const double r = s->q[0][n];
    const double u0 = s->q[1][n] / r, u1 = s->q[2][n] / r, u2 = s->q[3][n] / r;
    s->u[0][n] = u0;
    s->u[1][n] = u1;
    s->u[2][n] = u2;
    s->p[n] = (g - 1) * (s->q[4][n] - 0.5 * r * u0 * u0 - 0.5 * r * u1 * u1 - 0.5 * r * u2 * u2);
    s->a[n] = sqrt(g * s->p[n] / r);
  }
  FOR3(-2, N0 + 2, -2, N1 + 2, -2, N2 + 2) {
    const size_t n = I3(s, i, j, k);
    s->T[n] = M * M * g * s->p[n] / s->q[0][n];
    s->mu[n] = s->c.visc_pow > 0.0 ? pow(s->T[n], s->c.visc_pow) /* turbulent_channel.py:30 */
                                    : (ST + 1.0) * pow(s->T[n], 1.5) / (ST + s->T[n]);
  }
}

/* Modified Ducros sensor with the metric (shock_sensors.py:12-49 with metriceq, as generated for
 * transitional_SBLI.py): on the interior, with the x0 and x1 closures and d/dx1 = D11 d/dxi1,
 * theta = (1/2 - 1/2 tanh(250 div + 2.5)) div^2 / (eps + |curl u|^2 + div^2); 0 elsewhere. */
static void ducros_sensor(s3_t *s) {
  FOR3(0, N0, 0, N1, 0, N2) {
    const size_t n = I3(s, i, j, k);
    const double D = s->D11[j + H];
    double du[3][3];
    for (int c = 0; c < 3; ++c) {
      du[c][0] = d1c(s, s->u[c], i, j, k, 0);
      du[c][1] = D * d1c(s, s->u[c], i, j, k, 1);
      du[c][2] = d1c(s, s->u[c], i, j, k, 2);
    }
    const double div = du[0][0] + du[1][1] + du[2][2];
    const double w0 = du[2][1] - du[1][2], w1 = du[0][2] - du[2][0], w2 = du[1][0] - du[0][1];
    s->theta[n] = (0.5 - 0.5 * tanh(250.0 * div + 2.5)) * (div * div) /
                  (s->c.sensor_eps + w0 * w0 + w1 * w1 + w2 * w2 + div * div);
  }
}

/* TENO cut-off at the interface whose left point is n (teno.py:430-443) */
static double teno_cutoff(const s3_t *s, size_t n) {
  if (!s->c.teno_adaptive) return s->c.teno_ct;
  const double th = s->theta[n];
  return pow(10.0, -floor(s->c.teno_a1 - s->c.teno_a2 * (-pow(1 - th, 4) * (4 * th + 1) + 1)));
}

/* Body force of the continuity equation at the iteration `it` (transitional_SBLI.py:80-89) */
static void body_force(s3_t *s, int it) {
  if (s->c.bf_A == 0.0) return;
  const double st = sin(s->c.dt * s->c.bf_omega * it);
  FOR3(0, N0, 0, N1, 0, N2) {
    const double x0 = s->c.delta[0] * i, x1 = s->x1[j + H], x2 = s->c.delta[2] * k;
    s->res[0][I3(s, i, j, k)] += s->c.bf_A * exp(-(x0 - s->c.bf_xF) * (x0 - s->c.bf_xF) -
                                                 (x1 - s->c.bf_yF) * (x1 - s->c.bf_yF)) *
                                 st * cos(s->c.bf_bta * x2);
  }
}

/* The channel's constant forcing (turbulent_channel.py:15-16): -c_i in the momentum equations,
 * -c_j u_j in the energy equation. */
static void forcing(s3_t *s) {
  const double *f = s->c.force;
  if (f[0] == 0.0 && f[1] == 0.0 && f[2] == 0.0) return;
  FOR3(0, N0, 0, N1, 0, N2) {
    const size_t c = I3(s, i, j, k);
    for (int d = 0; d < 3; ++d) s->res[1 + d][c] -= f[d];
    s->res[4][c] -= f[0] * s->u[0][c] + f[1] * s->u[1][c] + f[2] * s->u[2][c];
  }
}

/* Characteristic fluxes in direction dir (Roe average, the Cartesian 3D eigensystem: the block's
 * metric is diagonal and enters the residual only), TENO5 / WENO5-JS / WENO5-Z / TENO6, and the
 * residual R = -(F_i - F_{i-1})/delta0 - D11 (G_j - G_{j-1})/delta1 - (H_k - H_{k-1})/delta2
 * (shock_capturing.py:21-34, opensblifunctions.py:658-676). */
static void residual_flux(s3_t *s) {
  const double g = s->c.gama;
  const int n[3] = {N0, N1, N2};
  if (s->c.teno_adaptive) ducros_sensor(s);
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) s->res[v][I3(s, i, j, k)] = 0.0;
  for (int dir = 0; dir < 3; ++dir) {
    const size_t o = dir == 0 ? 1 : dir == 1 ? (size_t)s->px : (size_t)s->px * s->py;
    int lo[3] = {0, 0, 0};
    lo[dir] = -1;
    FOR3(lo[0], n[0], lo[1], n[1], lo[2], n[2]) {
      const size_t c = I3(s, i, j, k);
      const double rl = s->q[0][c], rr = s->q[0][c + o];
      const double sl = sqrt(rl), sr = sqrt(rr);
      const double ar = sqrt(rl * rr), inv = 1.0 / (sl + sr);
      double au[3];
      for (int d = 0; d < 3; ++d) au[d] = inv * (sl * s->u[d][c] + sr * s->u[d][c + o]);
      const double Hh = inv * ((s->p[c] + s->q[4][c]) / sl + (s->p[c + o] + s->q[4][c + o]) / sr);
      const double aa = sqrt((g - 1) * (Hh - 0.5 * (au[0] * au[0] + au[1] * au[1] + au[2] * au[2])));
      double L[5][5], R[5][5];
      osbo_eigensystem3(dir, ar, au[0], au[1], au[2], aa, g, L, R);
      double CF[5][6], CS[5][6], lam[5] = {0, 0, 0, 0, 0};
      for (int t = 0; t < 6; ++t) {
        const size_t m = c + (size_t)((long)(t - 2) * (long)o);
        const double un = s->u[dir][m];
        double F[5], Q[5];
        for (int v = 0; v < 5; ++v) Q[v] = s->q[v][m];
        F[0] = s->q[1 + dir][m];
        for (int d = 0; d < 3; ++d) F[1 + d] = s->q[1 + d][m] * un + (d == dir ? s->p[m] : 0.0);
        F[4] = (s->p[m] + s->q[4][m]) * un;
        for (int r = 0; r < 5; ++r) {
          double cf = 0, cs = 0;
          for (int v = 0; v < 5; ++v) {
            cf += L[r][v] * F[v];
            cs += L[r][v] * Q[v];
          }
          CF[r][t] = cf;
          CS[r][t] = cs;
        }
        const double ev[5] = {fabs(un), fabs(un), fabs(un), fabs(un + s->a[m]), fabs(un - s->a[m])};
        for (int r = 0; r < 5; ++r) lam[r] = fmax(lam[r], ev[r]);
      }
      double rec[5];
      for (int r = 0; r < 5; ++r) {
        double fp[5], fm[5];
        for (int t = 0; t < 5; ++t) {
          fp[t] = CF[r][t] + lam[r] * CS[r][t];
          fm[t] = CF[r][t + 1] - lam[r] * CS[r][t + 1];
        }
        if (s->c.conv == OSBO_CONV_TENO6) {
          double gp[6], gm[6];
          for (int t = 0; t < 6; ++t) {
            gp[t] = CF[r][t] + lam[r] * CS[r][t];
            gm[t] = CF[r][t] - lam[r] * CS[r][t];
          }
          rec[r] = osbo_side_teno6(gp, 1, s->c.teno_eps, teno_cutoff(s, c)) +
                   osbo_side_teno6(gm, 0, s->c.teno_eps, teno_cutoff(s, c));
        } else if (s->c.conv == OSBO_CONV_WENO5JS || s->c.conv == OSBO_CONV_WENO5Z) {
          const int z = s->c.conv == OSBO_CONV_WENO5Z;
          rec[r] = osbo_side_weno5_plus(fp, z) + osbo_side_weno5_minus(fm, z);
        } else {
          const double fmr[5] = {fm[4], fm[3], fm[2], fm[1], fm[0]}; /* points i+3 .. i-1 */
          rec[r] = osbo_side_teno5(fp, s->c.teno_eps, teno_cutoff(s, c)) +
                   osbo_side_teno5(fmr, s->c.teno_eps, teno_cutoff(s, c));
        }
      }
      for (int v = 0; v < 5; ++v) {
        double fl = 0;
        for (int r = 0; r < 5; ++r) fl += R[v][r] * rec[r];
        s->flux[v][c] = fl;
      }
    }
    FOR3(0, N0, 0, N1, 0, N2) {
      const size_t c = I3(s, i, j, k);
      for (int v = 0; v < 5; ++v) {
        const double d = (s->flux[v][c] - s->flux[v][c - o]) / s->c.delta[dir];
        s->res[v][c] -= dir == 1 ? d * s->D11[j + H] : d;
      }
    }
  }
}

/* Viscous and heat-flux terms with Sutherland viscosity in the stretched metric (as
 * osb_oracle2d.c, three components): d/dx1 = D11 d/dxi1, d2/dx1^2 = D11^2 d2/dxi1^2 + D11 SD111
 * d/dxi1; mixed derivatives nest first derivatives, the inner x0 (or x2) derivative evaluated over
 * the extended range of the outer axis. */
static void residual_viscous(s3_t *s) {
  const double Re = s->c.Re;
  const double kap = 1.0 / ((s->c.gama - 1) * s->c.Minf * s->c.Minf * s->c.Pr * Re);
  for (int a = 0; a < 3; ++a) {
    FOR3(0, N0, -2, N1 + 2, -2, N2 + 2) s->wk[a][I3(s, i, j, k)] = d1c(s, s->u[a], i, j, k, 0);
    FOR3(0, N0, -2, N1 + 2, 0, N2) s->wz[a][I3(s, i, j, k)] = d1c(s, s->u[a], i, j, k, 2);
  }
  FOR3(0, N0, 0, N1, 0, N2) {
    const size_t c = I3(s, i, j, k);
    const double D = s->D11[j + H], S = s->SD111[j + H], mu = s->mu[c];
    double gr[3][3], h[3][3][3];
    for (int a = 0; a < 3; ++a) {
      const double fy = d1c(s, s->u[a], i, j, k, 1);
      gr[a][0] = s->wk[a][c];
      gr[a][1] = D * fy;
      gr[a][2] = s->wz[a][c];
      h[a][0][0] = d2c(s, s->u[a], i, j, k, 0);
      h[a][1][1] = D * D * d2c(s, s->u[a], i, j, k, 1) + D * S * fy;
      h[a][2][2] = d2c(s, s->u[a], i, j, k, 2);
      h[a][0][1] = h[a][1][0] = D * d1c(s, s->wk[a], i, j, k, 1);
      h[a][0][2] = h[a][2][0] = d1c(s, s->wk[a], i, j, k, 2);
      h[a][1][2] = h[a][2][1] = D * d1c(s, s->wz[a], i, j, k, 1);
    }
    const double mug[3] = {d1c(s, s->mu, i, j, k, 0), D * d1c(s, s->mu, i, j, k, 1), d1c(s, s->mu, i, j, k, 2)};
    const double Tg[3] = {d1c(s, s->T, i, j, k, 0), D * d1c(s, s->T, i, j, k, 1), d1c(s, s->T, i, j, k, 2)};
    const double Tlap = d2c(s, s->T, i, j, k, 0) + D * D * d2c(s, s->T, i, j, k, 1) +
                        D * S * d1c(s, s->T, i, j, k, 1) + d2c(s, s->T, i, j, k, 2);
    const double div = gr[0][0] + gr[1][1] + gr[2][2];
    double tau[3][3], dtau[3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) tau[a][b] = mu / Re * (gr[a][b] + gr[b][a] - (a == b ? 2.0 / 3.0 * div : 0.0));
    for (int a = 0; a < 3; ++a) {
      double v = 0.0;
      for (int b = 0; b < 3; ++b) v += mug[b] * (gr[a][b] + gr[b][a] - (a == b ? 2.0 / 3.0 * div : 0.0)) / Re;
      const double lap = h[a][0][0] + h[a][1][1] + h[a][2][2];
      const double ddiv = h[0][a][0] + h[1][a][1] + h[2][a][2];
      v += mu / Re * (lap + ddiv / 3.0);
      dtau[a] = v;
      s->res[1 + a][c] += v;
    }
    double e = kap * (mu * Tlap + mug[0] * Tg[0] + mug[1] * Tg[1] + mug[2] * Tg[2]);
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 3; ++b) e += tau[a][b] * gr[a][b];
      e += s->u[a][c] * dtau[a];
    }
    s->res[4][c] += e;
  }
}

static void load_padded(s3_t *s, const double *q) {
  const int hp = 4, pxo = N0 + 2 * hp, pyo = N1 + 2 * hp, pzo = N2 + 2 * hp;
  for (int v = 0; v < 5; ++v)
    FOR3(-hp, N0 + hp, -hp, N1 + hp, -hp, N2 + hp)
  s->q[v][I3(s, i, j, k)] = q[(((size_t)v * pzo + (size_t)(k + hp)) * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)];
}

int osbo3w_run(const osbo3w_cfg *cfg, double *q, int nsteps) {
  s3_t st, *s = &st;
  if (s3_init(s, cfg)) return -1;
  load_padded(s, q);
  metrics(s);
  for (int it = 0; it < nsteps; ++it) {
    apply_bcs(s);
    for (int stg = 0; stg < 3; ++stg) {
      constituent(s);
      residual_flux(s);
      forcing(s);
      body_force(s, it);
      residual_viscous(s);
      /* RungeKuttaLS (rk_LS.py:155-166): du = A du + dt R; q = q + B du */
      for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) {
          const size_t c = I3(s, i, j, k);
          s->du[v][c] = cfg->dt * s->res[v][c] + cfg->rkA[stg] * s->du[v][c];
          s->q[v][c] = cfg->rkB[stg] * s->du[v][c] + s->q[v][c];
        }
      apply_bcs(s);
    }
  }
  const int hp = 4, pxo = N0 + 2 * hp, pyo = N1 + 2 * hp, pzo = N2 + 2 * hp;
  for (int v = 0; v < 5; ++v)
    FOR3(-hp, N0 + hp, -hp, N1 + hp, -hp, N2 + hp)
  q[(((size_t)v * pzo + (size_t)(k + hp)) * pyo + (size_t)(j + hp)) * pxo + (size_t)(i + hp)] = s->q[v][I3(s, i, j, k)];
  s3_free(s);
  return 0;
}

int osbo3w_residual(const osbo3w_cfg *cfg, const double *q, double *r) {
  s3_t st, *s = &st;
  if (s3_init(s, cfg)) return -1;
  load_padded(s, q);
  metrics(s);
  apply_bcs(s);
  constituent(s);
  residual_flux(s);
  forcing(s);
  body_force(s, 0);
  residual_viscous(s);
  size_t m = 0;
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) r[m++] = s->res[v][I3(s, i, j, k)];
  s3_free(s);
  return 0;
}
