/* osb_oracle1d.c -- CPU restatement (FP64) of the generated per-timestep algorithm for a 1D Euler
 * block: apps/Sod_shock_tube/Sod_shock_tube.py (LLFTeno(5), RoeAverage) and apps/shu_osher/shu_osher.py
 * (LLFWeno(5, 'Z')), RungeKuttaLS(3), Dirichlet faces at both ends.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle).  See osb_oracle.h.
 *
 * Kernel order (algorithm.py:384-477): iter { BCs; stage { CRs u0, p, a over -3..n+4; characteristic
 * flux at the interfaces -1..n-1; residual R = -(F_i - F_{i-1})/delta0; LS-RK3 update; BCs } }.
 * The characteristic system is the reference's 1D one (physical_models/euler_eigensystem.py:57-76):
 * waves u-a, u, u+a, REV = [[1,1,1],[u-a,u,u+a],[H-ua,u^2/2,H+ua]], H = a^2/(gama-1) + u^2/2, and LEV
 * its inverse, evaluated from the interface's averaged u and a (averaging.py: Roe or simple).
 * Arrays carry a 5-point halo; the state exchanged with callers carries a 4-point halo.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "osb_oracle.h"

#define H 5

double osbo_side_weno5_plus(const double f[5], int z);
double osbo_side_weno5_minus(const double g[5], int z);
double osbo_side_teno6(const double g[6], int plus, double eps, double CT);
double osbo_side_teno5(const double f[5], double eps, double CT);

typedef struct {
  osbo1d_cfg c;
  int px;
  double *q[3], *du[3], *res[3], *flux[3], *u, *p, *a;
} s1_t;

#define N0 (s->c.n0)
#define IX(i) ((size_t)((i) + H))

static int s1_init(s1_t *s, const osbo1d_cfg *cfg) {
  memset(s, 0, sizeof(*s));
  s->c = *cfg;
  if (cfg->n0 < 8) return -1;
  s->px = cfg->n0 + 2 * H;
  for (int v = 0; v < 3; ++v) {
    s->q[v] = (double *)calloc(s->px, sizeof(double));
    s->du[v] = (double *)calloc(s->px, sizeof(double));
    s->res[v] = (double *)calloc(s->px, sizeof(double));
    s->flux[v] = (double *)calloc(s->px, sizeof(double));
  }
  s->u = (double *)calloc(s->px, sizeof(double));
  s->p = (double *)calloc(s->px, sizeof(double));
  s->a = (double *)calloc(s->px, sizeof(double));
  return 0;
}

static void s1_free(s1_t *s) {
  for (int v = 0; v < 3; ++v) {
    free(s->q[v]);
    free(s->du[v]);
    free(s->res[v]);
    free(s->flux[v]);
  }
  free(s->u);
  free(s->p);
  free(s->a);
}

/* DirichletBC (dirichlet.py:6-41): side 0 sets the points -3..0, side 1 the points n-1..n+3 to the
 * face's state; ExtrapolationBC order 0 (extrapolation.py:8-58) on side 1: n-1..n+3 take n-2. */
static void apply_bcs(s1_t *s) {
  for (int i = -3; i <= 0; ++i)
    for (int v = 0; v < 3; ++v) s->q[v][IX(i)] = s->c.face[0][v];
  for (int i = N0 - 1; i < N0 + 4; ++i)
    for (int v = 0; v < 3; ++v) s->q[v][IX(i)] = s->c.bc1 ? s->q[v][IX(N0 - 2)] : s->c.face[1][v];
}

/* Constituent relations (Sod_shock_tube.py:25-27) over -3..n+4 */
static void constituent(s1_t *s) {
  const double g = s->c.gama;
  for (int i = -3; i < N0 + 4; ++i) {
    const size_t n = IX(i);
    const double r = s->q[0][n];
    s->u[n] = s->q[1][n] / r;
    s->p[n] = (g - 1) * (s->q[2][n] - 0.5 * r * s->u[n] * s->u[n]);
    s->a[n] = sqrt(g * s->p[n] / r);
  }
}

/* The characteristic flux at the interface i+1/2 for i = -1..n-1 (shock_capturing.py:21-34) and the
 * residual. */
static void residual(s1_t *s) {
  const double g = s->c.gama, gm1 = g - 1;
  for (int i = -1; i < N0; ++i) {
    const size_t c = IX(i);
    double u, a;
    if (s->c.simple_avg) { /* SimpleAverage (averaging.py:31-59) */
      u = 0.5 * (s->u[c] + s->u[c + 1]);
      a = 0.5 * (s->a[c] + s->a[c + 1]);
    } else { /* RoeAverage (averaging.py:62-114) */
      const double sl = sqrt(s->q[0][c]), sr = sqrt(s->q[0][c + 1]), inv = 1.0 / (sl + sr);
      u = inv * (sl * s->u[c] + sr * s->u[c + 1]);
      const double Hh = inv * ((s->p[c] + s->q[2][c]) / sl + (s->p[c + 1] + s->q[2][c + 1]) / sr);
      a = sqrt(gm1 * (Hh - 0.5 * u * u));
    }
    const double ia = 1.0 / a, Hs = a * a / gm1 + 0.5 * u * u;
    /* LEV: the inverse of REV (rows: u-a, u, u+a) */
    double L[3][3];
    L[0][0] = 0.25 * u * ia * (gm1 * u * ia + 2.0);
    L[0][1] = -0.5 * ia * (gm1 * u * ia + 1.0);
    L[0][2] = 0.5 * gm1 * ia * ia;
    L[1][0] = 1.0 - 0.5 * gm1 * u * u * ia * ia;
    L[1][1] = gm1 * u * ia * ia;
    L[1][2] = -gm1 * ia * ia;
    L[2][0] = 0.25 * u * ia * (gm1 * u * ia - 2.0);
    L[2][1] = -0.5 * ia * (gm1 * u * ia - 1.0);
    L[2][2] = 0.5 * gm1 * ia * ia;
    double CF[3][6], CS[3][6], lam[3] = {0, 0, 0};
    for (int t = 0; t < 6; ++t) {
      const size_t m = IX(i + t - 2);
      const double un = s->u[m];
      const double F[3] = {s->q[1][m], s->q[1][m] * un + s->p[m], (s->p[m] + s->q[2][m]) * un};
      for (int r = 0; r < 3; ++r) {
        CF[r][t] = L[r][0] * F[0] + L[r][1] * F[1] + L[r][2] * F[2];
        CS[r][t] = L[r][0] * s->q[0][m] + L[r][1] * s->q[1][m] + L[r][2] * s->q[2][m];
      }
      const double ev[3] = {fabs(s->a[m] - un), fabs(un), fabs(s->a[m] + un)};
      for (int r = 0; r < 3; ++r) lam[r] = fmax(lam[r], ev[r]);
    }
    double rec[3];
    for (int r = 0; r < 3; ++r) {
      double fp[5], fm[5];
      for (int t = 0; t < 5; ++t) {
        fp[t] = CF[r][t] + lam[r] * CS[r][t];
        fm[t] = CF[r][5 - t] - lam[r] * CS[r][5 - t];
      }
      if (s->c.conv == OSBO_CONV_WENO5JS || s->c.conv == OSBO_CONV_WENO5Z) {
        double gm[5];
        for (int t = 0; t < 5; ++t) gm[t] = CF[r][t + 1] - lam[r] * CS[r][t + 1];
        const int z = s->c.conv == OSBO_CONV_WENO5Z;
        rec[r] = osbo_side_weno5_plus(fp, z) + osbo_side_weno5_minus(gm, z);
      } else if (s->c.conv == OSBO_CONV_TENO6) {
        double gp[6], gm[6];
        for (int t = 0; t < 6; ++t) {
          gp[t] = CF[r][t] + lam[r] * CS[r][t];
          gm[t] = CF[r][t] - lam[r] * CS[r][t];
        }
        rec[r] = osbo_side_teno6(gp, 1, s->c.teno_eps, s->c.teno_ct) + osbo_side_teno6(gm, 0, s->c.teno_eps, s->c.teno_ct);
      } else {
        rec[r] = osbo_side_teno5(fp, s->c.teno_eps, s->c.teno_ct) + osbo_side_teno5(fm, s->c.teno_eps, s->c.teno_ct);
      }
    }
    s->flux[0][c] = rec[0] + rec[1] + rec[2];
    s->flux[1][c] = (u - a) * rec[0] + u * rec[1] + (u + a) * rec[2];
    s->flux[2][c] = (Hs - u * a) * rec[0] + 0.5 * u * u * rec[1] + (Hs + u * a) * rec[2];
  }
  for (int i = 0; i < N0; ++i)
    for (int v = 0; v < 3; ++v) s->res[v][IX(i)] = -(s->flux[v][IX(i)] - s->flux[v][IX(i - 1)]) / s->c.delta0;
}

static void load(s1_t *s, const double *q) {
  const int hp = 4, pxo = N0 + 2 * hp;
  for (int v = 0; v < 3; ++v)
    for (int i = -hp; i < N0 + hp; ++i) s->q[v][IX(i)] = q[(size_t)v * pxo + (size_t)(i + hp)];
}

int osbo1d_run(const osbo1d_cfg *cfg, double *q, int nsteps) {
  s1_t st, *s = &st;
  if (s1_init(s, cfg)) return -1;
  load(s, q);
  for (int it = 0; it < nsteps; ++it) {
    apply_bcs(s);
    for (int stg = 0; stg < 3; ++stg) {
      constituent(s);
      residual(s);
      /* RungeKuttaLS (rk_LS.py:155-166): du = A du + dt R; q = q + B du */
      for (int v = 0; v < 3; ++v)
        for (int i = 0; i < N0; ++i) {
          s->du[v][IX(i)] = cfg->dt * s->res[v][IX(i)] + cfg->rkA[stg] * s->du[v][IX(i)];
          s->q[v][IX(i)] = cfg->rkB[stg] * s->du[v][IX(i)] + s->q[v][IX(i)];
        }
      apply_bcs(s);
    }
  }
  const int hp = 4, pxo = N0 + 2 * hp;
  for (int v = 0; v < 3; ++v)
    for (int i = -hp; i < N0 + hp; ++i) q[(size_t)v * pxo + (size_t)(i + hp)] = s->q[v][IX(i)];
  s1_free(s);
  return 0;
}

int osbo1d_residual(const osbo1d_cfg *cfg, const double *q, double *r) {
  s1_t st, *s = &st;
  if (s1_init(s, cfg)) return -1;
  load(s, q);
  apply_bcs(s);
  constituent(s);
  residual(s);
  for (int v = 0; v < 3; ++v)
    for (int i = 0; i < N0; ++i) r[(size_t)v * N0 + (size_t)i] = s->res[v][IX(i)];
  s1_free(s);
  return 0;
}
