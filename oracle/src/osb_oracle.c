/* osb_oracle.c -- CPU restatement (FP64) of OpenSBLI's generated per-timestep algorithm.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle).  See osb_oracle.h.
 *
 * The restatement follows the kernel list that the reference's TraditionalAlgorithmRK builds
 * (code_generation/algorithm/algorithm.py:384-477):
 *     iter { BC; save (RK only); stage { CRs; spatial residual; RK update; BC } }
 * with every array carrying a 5-point halo as the reference declares them
 * (schemes/spatial/scheme.py:47-60, code_generation/opsc.py:693-722).  It is written as plain
 * unfused array loops, one per reference kernel family, so that each piece can be read against the
 * generated code; speed is not a goal.
 */
#include "osb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define H 5 /* halo depth of every padded array, as in the reference */

typedef struct {
  osbo_cfg c;
  int nv;           /* number of conserved variables */
  int px, py, pz;   /* padded extents */
  int hz;           /* halo in z (0 in 2D) */
  size_t np;        /* padded points */
  double *q[5];     /* conserved, padded */
  double *qold[5];  /* RK old register (interior used) */
  double *res[5];   /* residual (interior used) */
  double *u[3], *p, *T, *a; /* constituent relations */
  double *wk[6];    /* scratch for nested derivatives */
  double *flux[5];  /* interface fluxes (WENO/TENO) */
  double *theta;    /* modified Ducros sensor (adaptive TENO), interior; 0 in the halos */
} st_t;

static inline size_t IX(const st_t *s, int i, int j, int k) {
  return (size_t)(i + H) + (size_t)s->px * ((size_t)(j + H) + (size_t)s->py * (size_t)(k + s->hz));
}

static double *alloc_pad(const st_t *s) { return (double *)calloc(s->np, sizeof(double)); }

static int st_init(st_t *s, const osbo_cfg *cfg) {
  memset(s, 0, sizeof(*s));
  s->c = *cfg;
  if (cfg->ndim != 3) return -1; /* this file restates the 3D path */
  s->nv = 5;
  s->hz = H;
  s->px = cfg->n[0] + 2 * H;
  s->py = cfg->n[1] + 2 * H;
  s->pz = cfg->n[2] + 2 * H;
  s->np = (size_t)s->px * s->py * s->pz;
  for (int v = 0; v < 5; ++v) {
    s->q[v] = alloc_pad(s);
    s->qold[v] = alloc_pad(s);
    s->res[v] = alloc_pad(s);
    s->flux[v] = alloc_pad(s);
  }
  for (int d = 0; d < 3; ++d) s->u[d] = alloc_pad(s);
  s->p = alloc_pad(s);
  s->T = alloc_pad(s);
  s->a = alloc_pad(s);
  for (int w = 0; w < 6; ++w) s->wk[w] = alloc_pad(s);
  s->theta = alloc_pad(s);
  return 0;
}

static void st_free(st_t *s) {
  for (int v = 0; v < 5; ++v) {
    free(s->q[v]);
    free(s->qold[v]);
    free(s->res[v]);
    free(s->flux[v]);
  }
  for (int d = 0; d < 3; ++d) free(s->u[d]);
  free(s->p);
  free(s->T);
  free(s->a);
  for (int w = 0; w < 6; ++w) free(s->wk[w]);
  free(s->theta);
}

#define N0 (s->c.n[0])
#define N1 (s->c.n[1])
#define N2 (s->c.n[2])
#define FOR3(i0, i1, j0, j1, k0, k1)          \
  for (int k = (k0); k < (k1); ++k)           \
    for (int j = (j0); j < (j1); ++j)         \
      for (int i = (i0); i < (i1); ++i)

/* ---------------------------------------------------------------------------------------------
 * Boundary conditions
 * ------------------------------------------------------------------------------------------- */

/* Periodic exchange (core/boundary_conditions/periodic.py:27-56, exchange.py:9-57): the reference
 * copies `depth` planes per side, x then y then z, each over the other axes' haloed range; the
 * result is a periodic wrap of every halo point, corners included. */
static void bc_periodic(st_t *s, int dir, int depth) {
  int n[3] = {N0, N1, N2};
  for (int v = 0; v < s->nv; ++v) {
    double *f = s->q[v];
    int lo[3] = {-depth, -depth, -depth}, hi[3] = {n[0] + depth, n[1] + depth, n[2] + depth};
    for (int side = 0; side < 2; ++side) {
      int l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]};
      if (side == 0) { l2[dir] = n[dir]; h2[dir] = n[dir] + depth; }
      else { l2[dir] = -depth; h2[dir] = 0; }
      FOR3(l2[0], h2[0], l2[1], h2[1], l2[2], h2[2]) {
        int src[3] = {i, j, k};
        src[dir] = side == 0 ? src[dir] - n[dir] : src[dir] + n[dir];
        f[IX(s, i, j, k)] = f[IX(s, src[0], src[1], src[2])];
      }
    }
  }
}

/* Symmetry condition (core/boundary_conditions/symmetry.py:23-50) for a Cartesian block: halo
 * point -t mirrors interior point +t about the boundary node; the momentum component normal to the
 * face changes sign; the boundary node itself is not modified.  Applied over the other axes'
 * range -depth..n+depth. */
static void bc_symmetry(st_t *s, int dir, int side, int depth) {
  int n[3] = {N0, N1, N2};
  int lo[3] = {-depth, -depth, -depth}, hi[3] = {n[0] + depth, n[1] + depth, n[2] + depth};
  lo[dir] = side == 0 ? 0 : n[dir] - 1;
  hi[dir] = lo[dir] + 1;
  int sgn = side == 0 ? -1 : 1;
  FOR3(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]) {
    for (int t = 1; t <= depth; ++t) {
      int to[3] = {i, j, k}, fr[3] = {i, j, k};
      to[dir] += sgn * t;
      fr[dir] -= sgn * t;
      for (int v = 0; v < 5; ++v) {
        double val = s->q[v][IX(s, fr[0], fr[1], fr[2])];
        if (v == 1 + dir) val = -1.0 * val;
        s->q[v][IX(s, to[0], to[1], to[2])] = val;
      }
    }
  }
}

/* exchanged depth: the central stencils reach 2 points, the characteristic fluxes (and the WENO filter) 3 */
static int halo_depth(const st_t *s) {
  return s->c.conv == OSBO_CONV_CENTRAL_SKEW && s->c.filter == OSBO_FILTER_NONE ? 2 : 3;
}

static void apply_bcs(st_t *s) {
  int depth = halo_depth(s);
  for (int d = 0; d < 3; ++d) {
    if (s->c.bc[d][0] == OSBO_BC_PERIODIC) {
      bc_periodic(s, d, depth);
    } else {
      bc_symmetry(s, d, 0, depth);
      bc_symmetry(s, d, 1, depth);
    }
  }
}

/* ---------------------------------------------------------------------------------------------
 * Constituent relations (taylor_green_vortex.py:30-32; the speed of sound as in
 * apps/katzer_SBLI/katzer_SBLI.py:21), evaluated over the whole padded range.
 * ------------------------------------------------------------------------------------------- */
static void constituent(st_t *s) {
  const double g = s->c.gama, M = s->c.Minf;
  for (size_t n = 0; n < s->np; ++n) {
    double rho = s->q[0][n];
    if (rho == 0.0) continue; /* never-written halo corner */
    double u0 = s->q[1][n] / rho, u1 = s->q[2][n] / rho, u2 = s->q[3][n] / rho;
    double p = (g - 1) * (s->q[4][n] - 0.5 * rho * u0 * u0 - 0.5 * rho * u1 * u1 - 0.5 * rho * u2 * u2);
    s->u[0][n] = u0;
    s->u[1][n] = u1;
    s->u[2][n] = u2;
    s->p[n] = p;
    s->T[n] = M * M * g * p / rho;
    s->a[n] = sqrt(g * p / rho);
  }
}

/* ---------------------------------------------------------------------------------------------
 * 4th-order central differences (core/opensblifunctions.py:485-521, scheme.py:81-85):
 *   d1 f = (f[-2]/12 - 2 f[-1]/3 + 2 f[1]/3 - f[2]/12) / delta
 *   d2 f = (-f[-2]/12 + 4 f[-1]/3 - 5 f[0]/2 + 4 f[1]/3 - f[2]/12) / delta^2
 * ------------------------------------------------------------------------------------------- */
static inline size_t stride(const st_t *s, int dir) {
  return dir == 0 ? 1 : dir == 1 ? (size_t)s->px : (size_t)s->px * s->py;
}
static inline double d1(const st_t *s, const double *f, size_t n, int dir) {
  size_t o = stride(s, dir);
  return ((1.0 / 12.0) * f[n - 2 * o] - (2.0 / 3.0) * f[n - o] + (2.0 / 3.0) * f[n + o] - (1.0 / 12.0) * f[n + 2 * o]) /
         s->c.delta[dir];
}
static inline double d2(const st_t *s, const double *f, size_t n, int dir) {
  size_t o = stride(s, dir);
  double h = s->c.delta[dir];
  return (-(1.0 / 12.0) * f[n - 2 * o] + (4.0 / 3.0) * f[n - o] - 2.5 * f[n] + (4.0 / 3.0) * f[n + o] -
          (1.0 / 12.0) * f[n + 2 * o]) / (h * h);
}

/* ---------------------------------------------------------------------------------------------
 * Convective terms, skew-symmetric central form (core/parsing.py:75-111 Skew, scheme.py:187-271):
 *   mass:   -Skew(rho u_j)         momentum: -Skew(rhou_i u_j) - d_i p
 *   energy: -Skew(rhoE u_j) - d_j(p u_j)
 * with Skew(phi u_j, x_j) = 1/2 [ d_j(phi u_j) + u_j d_j phi + phi d_j u_j ].
 * ------------------------------------------------------------------------------------------- */
static void residual_central_skew(st_t *s) {
  /* products phi*u_d for each direction are formed point-wise (the "Convective terms group d"
   * kernels) and differentiated along d */
  FOR3(0, N0, 0, N1, 0, N2) {
    size_t n = IX(s, i, j, k);
    double divu = 0.0;
    for (int d = 0; d < 3; ++d) divu += d1(s, s->u[d], n, d);
    for (int v = 0; v < 5; ++v) s->res[v][n] = 0.0;
    for (int v = 0; v < 5; ++v) {
      double r = 0.0;
      for (int d = 0; d < 3; ++d) {
        size_t o = stride(s, d);
        double prod[5];
        for (int t = -2; t <= 2; ++t) prod[t + 2] = s->q[v][n + t * o] * s->u[d][n + t * o];
        double dprod = ((1.0 / 12.0) * prod[0] - (2.0 / 3.0) * prod[1] + (2.0 / 3.0) * prod[3] -
                        (1.0 / 12.0) * prod[4]) / s->c.delta[d];
        r += dprod + s->u[d][n] * d1(s, s->q[v], n, d);
      }
      r += s->q[v][n] * divu;
      s->res[v][n] = -0.5 * r;
    }
    for (int d = 0; d < 3; ++d) s->res[1 + d][n] -= d1(s, s->p, n, d);
    double dpu = 0.0;
    for (int d = 0; d < 3; ++d) {
      size_t o = stride(s, d);
      double prod[5];
      for (int t = -2; t <= 2; ++t) prod[t + 2] = s->p[n + t * o] * s->u[d][n + t * o];
      dpu += ((1.0 / 12.0) * prod[0] - (2.0 / 3.0) * prod[1] + (2.0 / 3.0) * prod[3] - (1.0 / 12.0) * prod[4]) /
             s->c.delta[d];
    }
    s->res[4][n] -= dpu;
  }
}

/* ---------------------------------------------------------------------------------------------
 * Viscous and heat-flux terms with constant viscosity (taylor_green_vortex.py:18-19), expanded as
 * the reference's generated "Viscous residual" kernel does:
 *   momentum_i += (1/Re) [ lap u_i + 1/3 d_i (div u) ]
 *   energy     += kT lap T + tau_ij d_j u_i + u_i d_j tau_ij,  kT = 1/((gama-1) Minf^2 Pr Re)
 * Mixed derivatives nest first derivatives: d_j(d_i f) with the inner one evaluated over the halo
 * range of the outer direction (scheme.py:360-387).
 * ------------------------------------------------------------------------------------------- */
static void residual_viscous(st_t *s) {
  const double Re = s->c.Re;
  const double kT = 1.0 / ((s->c.gama - 1) * s->c.Minf * s->c.Minf * s->c.Pr * Re);
  /* inner first derivatives d_i u_c over the haloed range (-2..n+2 in every axis) */
  double *du[3][3];
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i) du[c][i] = alloc_pad(s);
  for (int c = 0; c < 3; ++c)
    for (int di = 0; di < 3; ++di) {
      int lo[3] = {0, 0, 0}, hi[3] = {N0, N1, N2};
      for (int a = 0; a < 3; ++a)
        if (a != di) { lo[a] = -2; hi[a] += 2; }
      FOR3(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]) {
        size_t n = IX(s, i, j, k);
        du[c][di][n] = d1(s, s->u[c], n, di);
      }
    }
  FOR3(0, N0, 0, N1, 0, N2) {
    size_t n = IX(s, i, j, k);
    double g[3][3];   /* g[c][d] = d_d u_c */
    double h2[3][3][3]; /* h2[c][a][b] = d_a d_b u_c */
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) g[c][d] = du[c][d][n];
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          if (a == b) h2[c][a][b] = d2(s, s->u[c], n, a);
          else {
            int inner = a < b ? a : b, outer = a < b ? b : a;
            h2[c][a][b] = d1(s, du[c][inner], n, outer);
          }
        }
    double divu = g[0][0] + g[1][1] + g[2][2];
    double tau[3][3], mom[3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) tau[i][j] = (g[i][j] + g[j][i] - (i == j ? 2.0 / 3.0 * divu : 0.0)) / Re;
    for (int i = 0; i < 3; ++i) {
      double lap = h2[i][0][0] + h2[i][1][1] + h2[i][2][2];
      double ddiv = h2[0][i][0] + h2[1][i][1] + h2[2][i][2];
      mom[i] = (lap + ddiv / 3.0) / Re;
      s->res[1 + i][n] += mom[i];
    }
    double lapT = d2(s, s->T, n, 0) + d2(s, s->T, n, 1) + d2(s, s->T, n, 2);
    double e = kT * lapT;
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) e += tau[i][j] * g[i][j];
      e += s->u[i][n] * mom[i];
    }
    s->res[4][n] += e;
  }
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i) free(du[c][i]);
}

/* ---------------------------------------------------------------------------------------------
 * Characteristic WENO5-JS with Roe averaging and local Lax-Friedrichs splitting.
 *   Roe average at i+1/2 (schemes/spatial/averaging.py:70-114).
 *   Eigensystem of the Euler equations for unit normal k (physical_models/euler_eigensystem.py:
 *   107-135): ev = (U,U,U,U+a,U-a), LEV/REV as given there.
 *   CF = LEV.F(stencil), CS = LEV.Q(stencil) at points i-2..i+3 (shock_capturing.py:357-398,
 *   464-495); lambda_r = max over the six points of |ev_r| from the point values (u, a) (:512-536);
 *   F+- = 1/2 (CF +- lambda CS).
 *   WENO5-JS (weno.py:70-205, 341-369): alpha_r = d_r/(1e-6 + beta_r)^2, omega_r = alpha_r/sum,
 *   or WENO5-Z (weno.py:283-331): alpha_r = d_r (1 + (tau/(1e-14 + beta_r))^2), tau = |beta_0 - beta_2|,
 *   candidate polynomials c_rj, optimal weights d = (3/10, 3/5, 1/10).
 *   Flux at i+1/2 = REV.(Fhat+ + Fhat-) (shock_capturing.py:418-448).
 * ------------------------------------------------------------------------------------------- */
/* The reference evaluates the split fluxes without their factor 1/2, f = CF +- lambda CS, and
 * folds the 1/2 into the smoothness indicators (1/4 of Jiang-Shu's, expanded as products) and into
 * the candidate stencils (1/2 of the usual c_rj).  The expressions below keep that form and term
 * order.  fp = f at points i-2..i+2 (upwind side), fm = f at points i-1..i+3. */
static double weno5_plus_w(const double f[5], int z, double *w) {
  const double b0 = 0.5 * f[2] * ((5.0 / 3.0) * f[2] - (31.0 / 6.0) * f[3] + (11.0 / 6.0) * f[4]) +
                    0.5 * f[3] * ((25.0 / 6.0) * f[3] - (19.0 / 6.0) * f[4]) + (1.0 / 3.0) * f[4] * f[4];
  const double b1 = 0.5 * f[1] * ((2.0 / 3.0) * f[1] - (13.0 / 6.0) * f[2] + (5.0 / 6.0) * f[3]) +
                    0.5 * f[2] * ((13.0 / 6.0) * f[2] - (13.0 / 6.0) * f[3]) + (1.0 / 3.0) * f[3] * f[3];
  const double b2 = 0.5 * f[0] * ((2.0 / 3.0) * f[0] + (11.0 / 6.0) * f[2]) +
                    0.5 * f[1] * (-(19.0 / 6.0) * f[0] + (25.0 / 6.0) * f[1] - (31.0 / 6.0) * f[2]) +
                    (5.0 / 6.0) * f[2] * f[2];
  double a0, a1, a2;
  if (z) {  /* WENO-Z (weno.py:283-331): d_r + d_r tau^2 / (beta_r + 1e-14)^2, tau = |beta_0 - beta_2| */
    const double t = fabs(b0 - b2);
    a0 = (3.0 / 10.0) + (3.0 / 10.0) * (t * t) / ((b0 + 1.0e-14) * (b0 + 1.0e-14));
    a1 = (3.0 / 5.0) + (3.0 / 5.0) * (t * t) / ((b1 + 1.0e-14) * (b1 + 1.0e-14));
    a2 = (1.0 / 10.0) + (1.0 / 10.0) * (t * t) / ((b2 + 1.0e-14) * (b2 + 1.0e-14));
  } else {
    a0 = (3.0 / 10.0) / ((b0 + 1e-6) * (b0 + 1e-6));
    a1 = (3.0 / 5.0) / ((b1 + 1e-6) * (b1 + 1e-6));
    a2 = (1.0 / 10.0) / ((b2 + 1e-6) * (b2 + 1e-6));
  }
  const double inv = 1.0 / (a0 + a1 + a2);
  if (w) { w[0] = a0 * inv; w[1] = a1 * inv; w[2] = a2 * inv; }
  return a0 * inv * ((1.0 / 6.0) * f[2] + (5.0 / 12.0) * f[3] - (1.0 / 12.0) * f[4]) +
         a1 * inv * (-(1.0 / 12.0) * f[1] + (5.0 / 12.0) * f[2] + (1.0 / 6.0) * f[3]) +
         a2 * inv * ((1.0 / 6.0) * f[0] - (7.0 / 12.0) * f[1] + (11.0 / 12.0) * f[2]);
}
static double weno5_plus(const double f[5], int z) { return weno5_plus_w(f, z, NULL); }
static double weno5_minus_w(const double g[5], int z, double *w) {
  /* g[0..4] = f at points i-1..i+3 (f1..f5 in the six-point numbering) */
  const double f1 = g[0], f2 = g[1], f3 = g[2], f4 = g[3], f5 = g[4];
  const double b0 = 0.5 * f3 * ((5.0 / 3.0) * f3 - (31.0 / 6.0) * f4 + (11.0 / 6.0) * f5) +
                    0.5 * f4 * ((25.0 / 6.0) * f4 - (19.0 / 6.0) * f5) + (1.0 / 3.0) * f5 * f5;
  const double b1 = 0.5 * f2 * ((2.0 / 3.0) * f2 - (13.0 / 6.0) * f3 + (5.0 / 6.0) * f4) +
                    0.5 * f3 * ((13.0 / 6.0) * f3 - (13.0 / 6.0) * f4) + (1.0 / 3.0) * f4 * f4;
  const double b2 = 0.5 * f1 * ((2.0 / 3.0) * f1 - (19.0 / 6.0) * f2 + (11.0 / 6.0) * f3) +
                    0.5 * f2 * ((25.0 / 6.0) * f2 - (31.0 / 6.0) * f3) + (5.0 / 6.0) * f3 * f3;
  double a0, a1, a2;
  if (z) {
    const double t = fabs(b0 - b2);
    a0 = (1.0 / 10.0) + (1.0 / 10.0) * (t * t) / ((b0 + 1.0e-14) * (b0 + 1.0e-14));
    a1 = (3.0 / 5.0) + (3.0 / 5.0) * (t * t) / ((b1 + 1.0e-14) * (b1 + 1.0e-14));
    a2 = (3.0 / 10.0) + (3.0 / 10.0) * (t * t) / ((b2 + 1.0e-14) * (b2 + 1.0e-14));
  } else {
    a0 = (1.0 / 10.0) / ((b0 + 1e-6) * (b0 + 1e-6));
    a1 = (3.0 / 5.0) / ((b1 + 1e-6) * (b1 + 1e-6));
    a2 = (3.0 / 10.0) / ((b2 + 1e-6) * (b2 + 1e-6));
  }
  const double inv = 1.0 / (a0 + a1 + a2);
  if (w) { w[0] = a0 * inv; w[1] = a1 * inv; w[2] = a2 * inv; }
  return a0 * inv * ((11.0 / 12.0) * f3 - (7.0 / 12.0) * f4 + (1.0 / 6.0) * f5) +
         a1 * inv * ((1.0 / 6.0) * f2 + (5.0 / 12.0) * f3 - (1.0 / 12.0) * f4) +
         a2 * inv * (-(1.0 / 12.0) * f1 + (5.0 / 12.0) * f2 + (1.0 / 6.0) * f3);
}

static double weno5_minus(const double g[5], int z) { return weno5_minus_w(g, z, NULL); }

/* TENO5 (schemes/spatial/teno.py:57-213, 407-465) with fixed cut-off C_T on one side of the split
 * flux, f[0..4] ordered from the far upwind point to the far downwind one: smoothness indicators of
 * the halved values (the splitting's 1/2, full Jiang-Shu form, teno.py:159-173), alpha_r =
 * (1 + tau5/(eps + beta_r))^6 with tau5 = |beta_0 - beta_2|, delta_r = 0 if alpha_r/sum(alpha) < C_T
 * else 1, omega_r = d_r delta_r / sum(d delta) with d = (0.55, 0.4, 0.05) for the central, downwind
 * and upwind candidates (teno.py:133; the same restatement as the 2D path's teno5_plus). */
static double teno5_side(const double f[5], double eps, double CT) {
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

/* TENO6 (schemes/spatial/teno.py:94-192, 216-234, 407-465) with fixed cut-off on one side of the
 * split flux.  g[0..5] are the split-flux values at points i-2 .. i+3 for either side; the four
 * stencils of the + side (fn_points, teno.py:100-105) are i-1..i+1, i..i+2, i-2..i and i..i+3, those of
 * the - side i..i+2, i-1..i+1, i+1..i+3 and i-2..i+1.  Indicators and candidates act on the halved values
 * (the splitting's 1/2, as the generated code writes them); the + side's fourth indicator carries the
 * reference's linear (unsquared) third-difference term (teno.py:175-176), the - side's the squared one.
 * tau6 = |beta_0/6 - 2 beta_1/3 + beta_2/6 - beta_3| (teno.py:229), alpha_r = (1 + tau6/(eps+beta_r))^6,
 * d = (231/500, 3/10, 27/500, 23/125). */
static double teno6_side(const double g[6], int plus, double eps, double CT) {
  double h[6];
  for (int t = 0; t < 6; ++t) h[t] = 0.5 * g[t];
  double b[4], p[4];
  if (plus) {
    b[0] = 0.25 * pow(h[1] - h[3], 2) + (13.0 / 12.0) * pow(h[1] - 2 * h[2] + h[3], 2);
    b[1] = (13.0 / 12.0) * pow(h[2] - 2 * h[3] + h[4], 2) + 0.25 * pow(3 * h[2] - 4 * h[3] + h[4], 2);
    b[2] = 0.25 * pow(h[0] - 4 * h[1] + 3 * h[2], 2) + (13.0 / 12.0) * pow(h[0] - 2 * h[1] + h[2], 2);
    b[3] = (1.0 / 36.0) * pow(-11 * h[2] + 18 * h[3] - 9 * h[4] + 2 * h[5], 2) +
           (13.0 / 12.0) * pow(2 * h[2] - 5 * h[3] + 4 * h[4] - h[5], 2) +
           (781.0 / 720.0) * (-h[2] + 3 * h[3] - 3 * h[4] + h[5]);
    p[0] = -(1.0 / 6.0) * h[1] + (5.0 / 6.0) * h[2] + (2.0 / 6.0) * h[3];
    p[1] = (2.0 / 6.0) * h[2] + (5.0 / 6.0) * h[3] - (1.0 / 6.0) * h[4];
    p[2] = (2.0 / 6.0) * h[0] - (7.0 / 6.0) * h[1] + (11.0 / 6.0) * h[2];
    p[3] = (3.0 / 12.0) * h[2] + (13.0 / 12.0) * h[3] - (5.0 / 12.0) * h[4] + (1.0 / 12.0) * h[5];
  } else {
    b[0] = 0.25 * pow(h[2] - h[4], 2) + (13.0 / 12.0) * pow(h[2] - 2 * h[3] + h[4], 2);
    b[1] = 0.25 * pow(h[1] - 4 * h[2] + 3 * h[3], 2) + (13.0 / 12.0) * pow(h[1] - 2 * h[2] + h[3], 2);
    b[2] = 0.25 * pow(3 * h[3] - 4 * h[4] + h[5], 2) + (13.0 / 12.0) * pow(h[3] - 2 * h[4] + h[5], 2);
    b[3] = (1.0 / 36.0) * pow(-2 * h[0] + 9 * h[1] - 18 * h[2] + 11 * h[3], 2) +
           (13.0 / 12.0) * pow(-h[0] + 4 * h[1] - 5 * h[2] + 2 * h[3], 2) +
           (781.0 / 720.0) * pow(-h[0] + 3 * h[1] - 3 * h[2] + h[3], 2);
    p[0] = (2.0 / 6.0) * h[2] + (5.0 / 6.0) * h[3] - (1.0 / 6.0) * h[4];
    p[1] = -(1.0 / 6.0) * h[1] + (5.0 / 6.0) * h[2] + (2.0 / 6.0) * h[3];
    p[2] = (11.0 / 6.0) * h[3] - (7.0 / 6.0) * h[4] + (2.0 / 6.0) * h[5];
    p[3] = (1.0 / 12.0) * h[0] - (5.0 / 12.0) * h[1] + (13.0 / 12.0) * h[2] + (3.0 / 12.0) * h[3];
  }
  const double tau = fabs(b[0] / 6.0 - 2.0 * b[1] / 3.0 + b[2] / 6.0 - b[3]);
  const double dw[4] = {231.0 / 500.0, 3.0 / 10.0, 27.0 / 500.0, 23.0 / 125.0};
  double a[4], sa = 0.0;
  for (int r = 0; r < 4; ++r) {
    a[r] = pow(1 + tau / (eps + b[r]), 6);
    sa += a[r];
  }
  double num = 0.0, den = 0.0;
  for (int r = 0; r < 4; ++r) {
    const double dl = CT > a[r] / sa ? 0.0 : 1.0;
    num += dw[r] * dl * p[r];
    den += dw[r] * dl;
  }
  return num / den;
}

static void eigensystem(int dir, double rho, double u0, double u1, double u2, double a, double g, double L[5][5],
                        double R[5][5]) {
  double k[3] = {0, 0, 0};
  k[dir] = 1.0;
  const double u[3] = {u0, u1, u2};
  const double phi = (g - 1) * 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
  const double th = k[0] * u0 + k[1] * u1 + k[2] * u2;
  const double al = rho / (a * sqrt(2.0)), bt = 1.0 / (rho * a * sqrt(2.0));
  const double a2 = a * a;
  /* rows 0..2: the three advective waves (euler_eigensystem.py:122 LEV) */
  L[0][0] = k[0] * (1 - phi / a2) - (k[2] * u1 - k[1] * u2) / rho;
  L[0][1] = k[0] * (g - 1) * u0 / a2;
  L[0][2] = k[0] * (g - 1) * u1 / a2 + k[2] / rho;
  L[0][3] = k[0] * (g - 1) * u2 / a2 - k[1] / rho;
  L[0][4] = -k[0] * (g - 1) / a2;
  L[1][0] = k[1] * (1 - phi / a2) - (k[0] * u2 - k[2] * u0) / rho;
  L[1][1] = k[1] * (g - 1) * u0 / a2 - k[2] / rho;
  L[1][2] = k[1] * (g - 1) * u1 / a2;
  L[1][3] = k[1] * (g - 1) * u2 / a2 + k[0] / rho;
  L[1][4] = -k[1] * (g - 1) / a2;
  L[2][0] = k[2] * (1 - phi / a2) - (k[1] * u0 - k[0] * u1) / rho;
  L[2][1] = k[2] * (g - 1) * u0 / a2 + k[1] / rho;
  L[2][2] = k[2] * (g - 1) * u1 / a2 - k[0] / rho;
  L[2][3] = k[2] * (g - 1) * u2 / a2;
  L[2][4] = -k[2] * (g - 1) / a2;
  L[3][0] = bt * (phi - th * a);
  L[4][0] = bt * (phi + th * a);
  for (int c = 0; c < 3; ++c) {
    L[3][1 + c] = -bt * ((g - 1) * u[c] - k[c] * a);
    L[4][1 + c] = -bt * ((g - 1) * u[c] + k[c] * a);
  }
  L[3][4] = bt * (g - 1);
  L[4][4] = bt * (g - 1);
  /* REV (euler_eigensystem.py:121) */
  R[0][0] = k[0]; R[0][1] = k[1]; R[0][2] = k[2]; R[0][3] = al; R[0][4] = al;
  R[1][0] = k[0] * u0; R[1][1] = k[1] * u0 - k[2] * rho; R[1][2] = k[2] * u0 + k[1] * rho;
  R[2][0] = k[0] * u1 + k[2] * rho; R[2][1] = k[1] * u1; R[2][2] = k[2] * u1 - k[0] * rho;
  R[3][0] = k[0] * u2 - k[1] * rho; R[3][1] = k[1] * u2 + k[0] * rho; R[3][2] = k[2] * u2;
  for (int c = 0; c < 3; ++c) {
    R[1 + c][3] = al * (u[c] + k[c] * a);
    R[1 + c][4] = al * (u[c] - k[c] * a);
  }
  R[4][0] = k[0] * phi / (g - 1) + rho * (k[2] * u1 - k[1] * u2);
  R[4][1] = k[1] * phi / (g - 1) + rho * (k[0] * u2 - k[2] * u0);
  R[4][2] = k[2] * phi / (g - 1) + rho * (k[1] * u0 - k[0] * u1);
  R[4][3] = al * ((phi + a2) / (g - 1) + th * a);
  R[4][4] = al * ((phi + a2) / (g - 1) - th * a);
}

/* Modified Ducros sensor on the interior (shock_sensors.py:12-49, the "ConstituentRelations CD" and
 * "ConstituentRelations evaluation" kernels): 4th-order central first derivatives of u_i,
 *   theta = (1/2 - 1/2 tanh(250 div + 2.5)) div^2 / (eps + |curl u|^2 + div^2);
 * the halos keep 0, so the TENO interfaces whose left point is a halo point take C_T = 10^-floor(a1). */
static void ducros_sensor(st_t *s) {
  FOR3(0, N0, 0, N1, 0, N2) {
    const size_t n = IX(s, i, j, k);
    double du[3][3];
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) du[c][d] = d1(s, s->u[c], n, d);
    const double div = du[0][0] + du[1][1] + du[2][2];
    const double w0 = du[2][1] - du[1][2], w1 = du[0][2] - du[2][0], w2 = du[1][0] - du[0][1];
    s->theta[n] = (0.5 - 0.5 * tanh(250.0 * div + 2.5)) * (div * div) /
                  (s->c.sensor_eps + w0 * w0 + w1 * w1 + w2 * w2 + div * div);
  }
}

/* TENO cut-off at the interface whose left point is n: fixed, or adapted (teno.py:430-443):
 * C_T = 10^-floor(a1 - a2 (1 - (1 - theta)^4 (4 theta + 1))) */
static double teno_cutoff3(const st_t *s, size_t n) {
  if (!s->c.teno_adaptive) return s->c.teno_ct;
  const double th = s->theta[n];
  return pow(10.0, -floor(s->c.teno_a1 - s->c.teno_a2 * (-pow(1 - th, 4) * (4 * th + 1) + 1)));
}

static void residual_weno(st_t *s) {
  const double g = s->c.gama;
  int n[3] = {N0, N1, N2};
  if (s->c.teno_adaptive) ducros_sensor(s);
  for (int v = 0; v < 5; ++v)
    FOR3(0, N0, 0, N1, 0, N2) s->res[v][IX(s, i, j, k)] = 0.0;
  for (int dir = 0; dir < 3; ++dir) {
    const size_t o = stride(s, dir);
    int lo[3] = {0, 0, 0}, hi[3] = {n[0], n[1], n[2]};
    lo[dir] = -1;
    FOR3(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]) {
      const size_t c = IX(s, i, j, k);
      /* Roe average between c and c+o */
      const double rl = s->q[0][c], rr = s->q[0][c + o];
      const double sl = sqrt(rl), sr = sqrt(rr);
      const double ar = sqrt(rl * rr), inv = 1.0 / (sl + sr);
      double au[3];
      for (int d = 0; d < 3; ++d) au[d] = inv * (sl * s->u[d][c] + sr * s->u[d][c + o]);
      const double Hh = inv * ((s->p[c] + s->q[4][c]) / sl + (s->p[c + o] + s->q[4][c + o]) / sr);
      const double aa = sqrt((g - 1) * (Hh - 0.5 * (au[0] * au[0] + au[1] * au[1] + au[2] * au[2])));
      double L[5][5], R[5][5];
      eigensystem(dir, ar, au[0], au[1], au[2], aa, g, L, R);
      /* characteristic flux and solution at the six points i-2..i+3 */
      double CF[5][6], CS[5][6];
      double lam[5] = {0, 0, 0, 0, 0};
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
          rec[r] = teno6_side(gp, 1, s->c.teno_eps, teno_cutoff3(s, c)) + teno6_side(gm, 0, s->c.teno_eps, teno_cutoff3(s, c));
        } else if (s->c.conv == OSBO_CONV_TENO5) {
          const double fmr[5] = {fm[4], fm[3], fm[2], fm[1], fm[0]};  /* points i+3 .. i-1 */
          rec[r] = teno5_side(fp, s->c.teno_eps, teno_cutoff3(s, c)) + teno5_side(fmr, s->c.teno_eps, teno_cutoff3(s, c));
        } else {
          rec[r] = weno5_plus(fp, s->c.conv == OSBO_CONV_WENO5Z) + weno5_minus(fm, s->c.conv == OSBO_CONV_WENO5Z);
        }
      }
      for (int v = 0; v < 5; ++v) {
        double fl = 0;
        for (int r = 0; r < 5; ++r) fl += R[v][r] * rec[r];
        s->flux[v][c] = fl;
      }
    }
    /* flux difference (opensblifunctions.py:575-593; shock_capturing.py:21-34) */
    FOR3(0, N0, 0, N1, 0, N2) {
      const size_t c = IX(s, i, j, k);
      for (int v = 0; v < 5; ++v) s->res[v][c] -= (s->flux[v][c] - s->flux[v][c - o]) / s->c.delta[dir];
    }
  }
}

/* ---------------------------------------------------------------------------------------------
 * WENO5 non-linear filter (filters/WENO_filter.py:15-339), applied after every full RK3 step with
 * dissipation_sensor='Constant' (kappa = 1):
 *   constituent relations of the filter (WENO_filter.py:134-168): inv_rho = 1/rho, u = rhou inv_rho,
 *     p = (g-1)(rhoE - 0.5 |rhou|^2 inv_rho), a = sqrt(g p inv_rho), over the padded range;
 *   per direction d, at interface i+1/2: the simple average of rho, u, a over points i, i+1
 *     (SimpleAverage([0, 1]), schemes/spatial/averaging.py), the Euler eigensystem of that state,
 *     CF = LEV.F with F = (rho u_d, rhou_c u_d + delta_cd p, (p + rhoE) u_d), CS = LEV.Q at i-2..i+3,
 *     lambda as for the LLF flux, WENO5-JS on f = CF +- lambda CS (weno.py:341-369), the weight
 *     sensor of each side r = sum_r |omega_r / d_r - 1|^4 / (9^4 + 2) (weno.py:436-452), rj = max of
 *     the two sides, Recon = rj (Recon - (CF_0 - 8 CF_1 + 37 CF_2 + 37 CF_3 - 8 CF_4 + CF_5)/60)
 *     (shock_capturing.py:399-412, 440-442), flux = REV.Recon;
 *   q += dt * shock_filter_control * Wall * kappa * (-sum_d (flux_d[i] - flux_d[i-1]) / delta_d)
 *     (WENO_filter.py:258-282), Wall = 1 away from wall faces (periodic blocks: everywhere).
 * ------------------------------------------------------------------------------------------- */
static double filter_side_sensor(const double w[3], const double inv_d[3]) {
  double num = 0.0;
  for (int r = 0; r < 3; ++r) num += pow(fabs(inv_d[r] * w[r] - 1.0), 4.0);
  return num / (pow(9.0, 4.0) + 2.0);
}

static void weno_filter(st_t *s) {
  const double g = s->c.gama;
  int n[3] = {N0, N1, N2};
  for (size_t m = 0; m < s->np; ++m) {
    const double rho = s->q[0][m];
    if (rho == 0.0) continue;
    const double ir = 1.0 / rho;
    for (int d = 0; d < 3; ++d) s->u[d][m] = s->q[1 + d][m] * ir;
    const double p = (g - 1) * (s->q[4][m] - 0.5 * (s->q[1][m] * s->q[1][m] + s->q[2][m] * s->q[2][m] +
                                                     s->q[3][m] * s->q[3][m]) * ir);
    s->p[m] = p;
    s->a[m] = sqrt(g * p * ir);
  }
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) s->res[v][IX(s, i, j, k)] = 0.0;
  static const double inv_dp[3] = {10.0 / 3.0, 5.0 / 3.0, 10.0}, inv_dm[3] = {10.0, 5.0 / 3.0, 10.0 / 3.0};
  for (int dir = 0; dir < 3; ++dir) {
    const size_t o = stride(s, dir);
    int lo[3] = {0, 0, 0}, hi[3] = {n[0], n[1], n[2]};
    lo[dir] = -1;
    FOR3(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]) {
      const size_t c = IX(s, i, j, k);
      const double ar = 0.5 * (s->q[0][c + o] + s->q[0][c]);
      const double aa = 0.5 * (s->a[c] + s->a[c + o]);
      double au[3];
      for (int d = 0; d < 3; ++d) au[d] = 0.5 * (s->u[d][c + o] + s->u[d][c]);
      double L[5][5], R[5][5];
      eigensystem(dir, ar, au[0], au[1], au[2], aa, g, L, R);
      double CF[5][6], CS[5][6];
      double lam[5] = {0, 0, 0, 0, 0};
      for (int t = 0; t < 6; ++t) {
        const size_t m = c + (size_t)((long)(t - 2) * (long)o);
        const double un = s->u[dir][m];
        double F[5], Q[5];
        for (int v = 0; v < 5; ++v) Q[v] = s->q[v][m];
        F[0] = s->q[0][m] * un;
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
        double fp[5], fm[5], wp[3], wm[3];
        for (int t = 0; t < 5; ++t) {
          fp[t] = CF[r][t] + lam[r] * CS[r][t];
          fm[t] = CF[r][t + 1] - lam[r] * CS[r][t + 1];
        }
        const double recon = weno5_plus_w(fp, 0, wp) + weno5_minus_w(fm, 0, wm);
        const double rj = fmax(filter_side_sensor(wp, inv_dp), filter_side_sensor(wm, inv_dm));
        const double central = (1.0 / 60.0) * (CF[r][0] - 8.0 * CF[r][1] + 37.0 * CF[r][2] + 37.0 * CF[r][3] -
                                               8.0 * CF[r][4] + CF[r][5]);
        rec[r] = rj * (recon - central);
      }
      for (int v = 0; v < 5; ++v) {
        double fl = 0;
        for (int r = 0; r < 5; ++r) fl += R[v][r] * rec[r];
        s->flux[v][c] = fl;
      }
    }
    FOR3(0, N0, 0, N1, 0, N2) {
      const size_t c = IX(s, i, j, k);
      for (int v = 0; v < 5; ++v) s->res[v][c] -= (s->flux[v][c] - s->flux[v][c - o]) / s->c.delta[dir];
    }
  }
  const double scale = s->c.dt * s->c.filter_control;
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) {
      const size_t c = IX(s, i, j, k);
      s->q[v][c] += scale * s->res[v][c];
    }
}

/* ---------------------------------------------------------------------------------------------
 * Time advance: 2-register RK3 (schemes/temporal/rk_sbli.py:51-61, 117-133):
 *   save: qold = q
 *   stage s: q = qold + dt*rknew[s]*R ; qold = qold + dt*rkold[s]*R
 * ------------------------------------------------------------------------------------------- */
static const double RKOLD[3] = {1.0 / 4.0, 3.0 / 20.0, 3.0 / 5.0};
static const double RKNEW[3] = {2.0 / 3.0, 5.0 / 12.0, 3.0 / 5.0};

static void residual(st_t *s) {
  constituent(s);
  if (s->c.conv == OSBO_CONV_CENTRAL_SKEW) residual_central_skew(s);
  else residual_weno(s);
  if (s->c.visc == OSBO_VISC_CONST) residual_viscous(s);
}

static double kinetic_energy(st_t *s) {
  double ke = 0;
  FOR3(0, N0, 0, N1, 0, N2) {
    size_t n = IX(s, i, j, k);
    double r = s->q[0][n];
    ke += 0.5 * (s->q[1][n] * s->q[1][n] + s->q[2][n] * s->q[2][n] + s->q[3][n] * s->q[3][n]) / r;
  }
  return ke / ((double)N0 * N1 * N2);
}

static void load_interior(st_t *s, const double *q) {
  size_t m = 0;
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) s->q[v][IX(s, i, j, k)] = q[m++];
}
static void store_interior(st_t *s, double *q, double **src) {
  size_t m = 0;
  for (int v = 0; v < 5; ++v) FOR3(0, N0, 0, N1, 0, N2) q[m++] = src[v][IX(s, i, j, k)];
}

int osbo_tgv_init(const osbo_cfg *cfg, double *q) {
  const int n0 = cfg->n[0], n1 = cfg->n[1], n2 = cfg->n[2];
  const size_t N = (size_t)n0 * n1 * n2;
  const double g = cfg->gama, M = cfg->Minf;
  for (int k = 0; k < n2; ++k)
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n0; ++i) {
        const double x0 = cfg->delta[0] * i, x1 = cfg->delta[1] * j, x2 = cfg->delta[2] * k;
        const double u0 = sin(x0) * cos(x1) * cos(x2), u1 = -sin(x1) * cos(x0) * cos(x2), u2 = 0.0;
        const double p = (0.0625 * cos(2.0 * x0) + 0.0625 * cos(2.0 * x1)) * (cos(2.0 * x2) + 2.0) + 1.0 / (M * M * g);
        const double r = M * M * g * p;
        const size_t m = (size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * k);
        q[0 * N + m] = r;
        q[1 * N + m] = r * u0;
        q[2 * N + m] = r * u1;
        q[3 * N + m] = r * u2;
        q[4 * N + m] = p / (g - 1) + 0.5 * r * (u0 * u0 + u1 * u1 + u2 * u2);
      }
  return 0;
}

int osbo_residual(const osbo_cfg *cfg, const double *q, double *r) {
  st_t s;
  if (st_init(&s, cfg)) return -1;
  load_interior(&s, q);
  apply_bcs(&s);
  residual(&s);
  store_interior(&s, r, s.res);
  st_free(&s);
  return 0;
}

int osbo_cutoff(const osbo_cfg *cfg, const double *q, double *ct) {
  if (!cfg->teno_adaptive) return -1;
  st_t st, *s = &st;
  if (st_init(s, cfg)) return -1;
  load_interior(s, q);
  apply_bcs(s);
  constituent(s);
  ducros_sensor(s);
  size_t m = 0;
  FOR3(0, N0, 0, N1, 0, N2) ct[m++] = teno_cutoff3(s, IX(s, i, j, k));
  st_free(s);
  return 0;
}

int osbo_run(const osbo_cfg *cfg, double *q, int nsteps, double *ke) {
  st_t s;
  if (st_init(&s, cfg)) return -1;
  load_interior(&s, q);
  if (ke) ke[0] = kinetic_energy(&s);
  for (int it = 0; it < nsteps; ++it) {
    apply_bcs(&s);
    for (int v = 0; v < 5; ++v) FOR3(0, s.c.n[0], 0, s.c.n[1], 0, s.c.n[2]) {
        size_t n = IX(&s, i, j, k);
        s.qold[v][n] = s.q[v][n];
      }
    for (int st = 0; st < 3; ++st) {
      residual(&s);
      const double dt = s.c.dt;
      for (int v = 0; v < 5; ++v) FOR3(0, s.c.n[0], 0, s.c.n[1], 0, s.c.n[2]) {
          size_t n = IX(&s, i, j, k);
          s.q[v][n] = dt * RKNEW[st] * s.res[v][n] + s.qold[v][n];
          s.qold[v][n] = dt * RKOLD[st] * s.res[v][n] + s.qold[v][n];
        }
      apply_bcs(&s);
    }
    if (s.c.filter == OSBO_FILTER_WENO5_CONSTANT) weno_filter(&s);
    if (ke) ke[it + 1] = kinetic_energy(&s);
  }
  store_interior(&s, q, s.q);
  st_free(&s);
  return 0;
}

/* The reconstruction sides, shared with the 2D restatement (osb_oracle2d.c). */
double osbo_side_weno5_plus(const double f[5], int z) { return weno5_plus(f, z); }
double osbo_side_weno5_minus(const double g[5], int z) { return weno5_minus(g, z); }
double osbo_side_teno6(const double g[6], int plus, double eps, double CT) { return teno6_side(g, plus, eps, CT); }
double osbo_side_teno5(const double f[5], double eps, double CT) { return teno5_side(f, eps, CT); }
void osbo_eigensystem3(int dir, double rho, double u0, double u1, double u2, double a, double g, double L[5][5],
                       double R[5][5]) {
  eigensystem(dir, rho, u0, u1, u2, a, g, L, R);
}
