// osb_2d.cu -- the 2D curvilinear wall-bounded path: metrics stretched in x1, TENO5 (or WENO5-JS)
// characteristic fluxes, Sutherland viscous terms with one-sided boundary closures, the
// low-storage RK3 update and the four face conditions of the shock/boundary-layer problem.
//
// Kernel list per RK stage (the generated loop, algorithm.py:384-477, for
// apps/katzer_SBLI/katzer_SBLI.py):
//   k2_prims   constituent relations u0, u1, p, a, T, mu (Sutherland) from the FP64 master; mixed:
//              also the FP32 working state
//   k2_sensor_ct (adaptive TENO only): modified Ducros sensor theta and the cut-off C_T per point
//   k2_flux<T, D, SCHEME> for D = x0, x1: interface fluxes + flux difference into R
//   k2_visc    viscous/heat-flux terms (shared-memory tiles), concurrent with the two flux kernels
//   k2_rk      R = x fluxes + x1 fluxes + viscous terms; LS-RK3: du = A du + dt R, q += B du (FP64)
//   k2_bc      the four face conditions on the FP64 master, one launch (inlet and outlet, then wall
//              and top: the generated order where it matters)
// A step starts with the face conditions and, mixed, ends with k2_to_state (the bound FP32 arrays
// current).
// Metrics (once, k2_metric_*): detJ = dx1/dxi1 with the closures, D11 = 1/detJ, halos mirrored about
// the boundary points, SD111 = dD11/dxi1 (equation_types/metric.py:37-234, 315-332).
#include <cmath>
#include <utility>

#include "osb_common.cuh"
#include "osb_cvt.cuh"
#include "osb_internal.h"
#include "osb_weno.cuh"  // the WENO5-Z and TENO6 sides (weno5_side, teno6_side) and the SCH_* scheme codes

namespace osb {

namespace {

template <typename T> __device__ __forceinline__ T rcp2(T x);
template <> __device__ __forceinline__ float rcp2<float>(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double rcp2<double>(double x) { return 1.0 / x; }
template <typename T> __device__ __forceinline__ T pow_t(T x, T y);
template <> __device__ __forceinline__ float pow_t<float>(float x, float y) { return powf(x, y); }
template <> __device__ __forceinline__ double pow_t<double>(double x, double y) { return pow(x, y); }

// ---- one-sided closures of the central first derivative.  G(o) reads the function at offset o
// along the axis, k is the point's index, n the axis size, cl the axis's Carpenter faces (bit 0: side
// 0, bit 1: side 1; the others are ReducedAccess); bit 2 marks a periodic axis (central everywhere),
// bits 3 and 4 a side 0 / side 1 without a closure (a symmetry face: central over its mirrored halos).
//  * ReducedAccess (reduced_access_scheme.py:34-83): the first two points of a face, 5-point stencils;
//  * Carpenter (Carpenter_scheme.py:61-102): the first four points, weights c_carp[r][m] of f(m) at
//    point r of a side-0 face, mirrored with the opposite sign on side 1.
// A point within reach of both faces takes the side-0 closure (its condition comes first).
__constant__ double c_carp_d[24];
__constant__ float c_carp_f[24];
template <typename T> __device__ __forceinline__ T carp_w(int i);
template <> __device__ __forceinline__ double carp_w<double>(int i) { return c_carp_d[i]; }
template <> __device__ __forceinline__ float carp_w<float>(int i) { return c_carp_f[i]; }

template <typename T, typename Gf> __device__ __forceinline__ T d1c(const Gf &G, int k, int n, int cl) {
  const int w0 = (cl & 8) ? 0 : (cl & 1) ? 4 : 2, w1 = (cl & 16) ? 0 : (cl & 2) ? 4 : 2;
  if (!(cl & 4) && (k < w0 || n - 1 - k < w1)) {
    const bool s0 = k < w0;
    if (s0 ? (cl & 1) : (cl & 2)) {
      const int r = s0 ? k : n - 1 - k;
      T v = T(0);
#pragma unroll
      for (int m = 0; m < 6; ++m) v += carp_w<T>(6 * r + m) * (s0 ? G(m - r) : G(r - m));
      return s0 ? v : -v;
    }
    if (s0 && k == 0)
      return T(-25.0 / 12.0) * G(0) + T(4) * G(1) - T(3) * G(2) + T(4.0 / 3.0) * G(3) - T(0.25) * G(4);
    if (s0) return T(-0.25) * G(-1) - T(5.0 / 6.0) * G(0) + T(1.5) * G(1) - T(0.5) * G(2) + T(1.0 / 12.0) * G(3);
    if (k == n - 1)
      return T(25.0 / 12.0) * G(0) - T(4) * G(-1) + T(3) * G(-2) - T(4.0 / 3.0) * G(-3) + T(0.25) * G(-4);
    return T(0.25) * G(1) + T(5.0 / 6.0) * G(0) - T(1.5) * G(-1) + T(0.5) * G(-2) - T(1.0 / 12.0) * G(-3);
  }
  return T(1.0 / 12.0) * G(-2) - T(2.0 / 3.0) * G(-1) + T(2.0 / 3.0) * G(1) - T(1.0 / 12.0) * G(2);
}
// second derivative: the same two-point closure in both schemes (second_der_coefficients); none on a
// periodic axis (cl bit 2)
template <typename T, typename Gf> __device__ __forceinline__ T d2c(const Gf &G, int k, int n, int cl = 0) {
  const bool s0 = !(cl & 12), s1 = !(cl & 20);  // side 0 / side 1 closed
  if (k == 0 && s0)
    return T(35.0 / 12.0) * G(0) - T(26.0 / 3.0) * G(1) + T(9.5) * G(2) - T(14.0 / 3.0) * G(3) + T(11.0 / 12.0) * G(4);
  if (k == 1 && s0)
    return T(11.0 / 12.0) * G(-1) - T(5.0 / 3.0) * G(0) + T(0.5) * G(1) + T(1.0 / 3.0) * G(2) - T(1.0 / 12.0) * G(3);
  if (k == n - 1 && s1)
    return T(35.0 / 12.0) * G(0) - T(26.0 / 3.0) * G(-1) + T(9.5) * G(-2) - T(14.0 / 3.0) * G(-3) + T(11.0 / 12.0) * G(-4);
  if (k == n - 2 && s1)
    return T(11.0 / 12.0) * G(1) - T(5.0 / 3.0) * G(0) + T(0.5) * G(-1) + T(1.0 / 3.0) * G(-2) - T(1.0 / 12.0) * G(-3);
  return T(-1.0 / 12.0) * G(-2) + T(4.0 / 3.0) * G(-1) - T(2.5) * G(0) + T(4.0 / 3.0) * G(1) - T(1.0 / 12.0) * G(2);
}

__device__ __forceinline__ int64_t g2(const Grid &g, int i, int j) { return g.off0 + (int64_t)i + (int64_t)j * g.sy; }

}  // namespace

// ---------------------------------------------------------------------------------------------
// metrics
// ---------------------------------------------------------------------------------------------
__global__ void k2_metric_d11(Grid g, const double *x1, double *D11, double inv_d1, int cly) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n0 || j >= g.n1) return;
  auto G = [&](int o) { return x1[g2(g, i, j + o)]; };
  const double detJ = inv_d1 * d1c<double>(G, j, g.n1, cly);
  D11[g2(g, i, j)] = 1.0 / detJ;
}

// mirror D11 into the halos: axis 0 then axis 1, sides 0 and 1 (3 points on side 0, 4 on side 1)
__global__ void k2_metric_halo(Grid g, double *D11, int axis, int hx, int hy) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (axis == 0) {
    const int j = t - hy;
    if (j >= g.n1 + hy) return;
    for (int k = 1; k <= 3; ++k) D11[g2(g, -k, j)] = D11[g2(g, k, j)];
    for (int k = 1; k <= 4 && k <= hx; ++k) D11[g2(g, g.n0 - 1 + k, j)] = D11[g2(g, g.n0 - 1 - k, j)];
  } else {
    const int i = t - hx;
    if (i >= g.n0 + hx) return;
    for (int k = 1; k <= 3; ++k) D11[g2(g, i, -k)] = D11[g2(g, i, k)];
    for (int k = 1; k <= 4 && k <= hy; ++k) D11[g2(g, i, g.n1 - 1 + k)] = D11[g2(g, i, g.n1 - 1 - k)];
  }
}

__global__ void k2_metric_sd(Grid g, const double *D11, double *SD111, double inv_d1, int cly) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n0 || j >= g.n1) return;
  auto G = [&](int o) { return D11[g2(g, i, j + o)]; };
  SD111[g2(g, i, j)] = inv_d1 * d1c<double>(G, j, g.n1, cly);
}

// ---------------------------------------------------------------------------------------------
// boundary conditions on the FP64 master state, x0 side 0, x0 side 1, x1 side 0, x1 side 1
// ---------------------------------------------------------------------------------------------
struct Q4 {
  double *v[4];
};

// Face conditions of the shock/boundary-layer block:
//  * InletPressureExtrapolateBC (core/boundary_conditions/inlet_pressure_extrapolate.py:11-66):
//    supersonic points at i = 0 take the halo state at i = -1; subsonic points keep their state and
//    the energy halos take rhoE(0);
//  * ExtrapolationBC, order 0 (core/boundary_conditions/extrapolation.py:8-58): the last point and
//    the halo points take the state of point n0-2;
//  * IsothermalWallBC (core/boundary_conditions/isothermal_wall.py:32-88): zero momentum at the
//    wall, wall energy from Twall, halo states mirrored with a linearly extrapolated temperature;
//  * DirichletBC with a piecewise state in x0 (katzer_SBLI.py:108-114): points j >= n1-1 take
//    state[1] where x0 = delta0 * i > x_switch and state[0] elsewhere.
struct Dir2 {
  double lo[4], hi[4];
};

// The four faces in one launch.  The inlet and outlet touch the columns -3..0 and n0-2..n0+hx (the
// outlet reads n0-2), the wall and the top face the rows -3..3 and n1-1..n1+hy (the wall reads rows
// 0..3); the generated order (inlet, outlet, wall, top) only matters where these meet: the wall reads
// the x-halo columns the inlet and outlet wrote, the outlet must read column n0-2 before the wall
// writes it, and at the corners the later face wins.  So block 0 applies the x faces of the rows
// -3..3 and n1-5..n1+hy (a symmetry top face reads rows n1-5..n1-2), then (after a barrier) the y
// faces of the columns -3..0 and n0-2..n0+hx;
// the other blocks apply the x faces of the rows between and the y faces of the columns between,
// which no other work item touches.  Each y-face column is three work items, one per wall halo
// point, so the FP64 divisions of a column run in parallel.
struct BC2Args {
  double gama, Minf, Twall, delta0, xs;
  int hx, hy;
  Dir2 st;
  // Euler blocks: Dirichlet x0 faces (constant states f0 on side 0, f1 on side 1) instead of the inlet
  // and the outlet; symmetry x1 faces instead of the wall (side 0) and the Dirichlet face (side 1)
  int dir0, dir1, sym0, sym1;
  double f0[4], f1[4];
  // viscous_shock_tube.py: adiabatic walls on the x0 faces and on x1 side 0
  int adi0, adi1, adiy0;
  // laminar_channel.py: periodic x0 (wrapped after the faces) and an isothermal wall on x1 side 1
  int per0, wall1;
};

// AdiabaticWallBC (adiabatic_wall.py, as generated for viscous_shock_tube.py) on one line across a face
// whose boundary point is b (index along the face normal) and interior lies on the side sg: zero
// momentum at b, T_w = (18 T_1 - 9 T_2 + 2 T_3)/11 over the first three interior points, rhoE_w =
// rho_w T_w / (gama Minf^2 (gama-1)); halo t mirrors interior t, rho and rhoE even, momentum odd
// (t = 1..nt; the other threads of the face write only halo points, which this point never reads).
template <typename At>
__device__ __forceinline__ void adia2_line(const Q4 &q, const BC2Args &a, At at, int bnd, int sg, int t0, int t1) {
  for (int t = t0; t <= t1; ++t) {
    const int64_t h = at(bnd - sg * t), m = at(bnd + sg * t);
    q.v[0][h] = q.v[0][m];
    q.v[1][h] = -q.v[1][m];
    q.v[2][h] = -q.v[2][m];
    q.v[3][h] = q.v[3][m];
  }
  if (t0 == 1) {
    const double gm1 = a.gama - 1.0, gM2 = a.gama * a.Minf * a.Minf;
    double T[4];
    for (int k = 1; k <= 3; ++k) {
      const int64_t m = at(bnd + sg * k);
      const double r = q.v[0][m];
      T[k] = gM2 * gm1 * (q.v[3][m] - 0.5 * (q.v[1][m] * q.v[1][m] + q.v[2][m] * q.v[2][m]) / r) / r;
    }
    const int64_t w = at(bnd);
    q.v[1][w] = 0.0;
    q.v[2][w] = 0.0;
    q.v[3][w] = (18.0 / 11.0 * T[1] - 9.0 / 11.0 * T[2] + 2.0 / 11.0 * T[3]) * q.v[0][w] / (gM2 * gm1);
  }
}

// inlet (i = 0 and its halo) and outlet (i >= n0-1) of row j, or the Dirichlet x0 faces
// (dirichlet.py:6-41: the boundary point and the halo take the face's state)
__device__ __forceinline__ void bc2_row(const Grid &g, const Q4 &q, const BC2Args &a, int j) {
  if (a.per0) return;  // the x0 exchange follows the faces (k2_wrap)
  if (a.adi0) {  // both x0 faces adiabatic (the 4-point halo of side 1 as generated)
    auto at = [&](int i) { return g2(g, i, j); };
    adia2_line(q, a, at, 0, 1, 1, 3);
    adia2_line(q, a, at, g.n0 - 1, -1, 1, 4);
    return;
  }
  if (a.dir0) {
    for (int i = -3; i <= 0; ++i)
      for (int v = 0; v < 4; ++v) q.v[v][g2(g, i, j)] = a.f0[v];
  } else {  // inlet
    const int64_t b = g2(g, 0, j), m1 = g2(g, -1, j);
    const double rhob = q.v[0][b];
    const double ub0 = fabs(q.v[1][b] / rhob), ub1 = fabs(q.v[2][b] / rhob);
    const double pb = (a.gama - 1) * (-0.5 * rhob * (ub0 * ub0 + ub1 * ub1) + q.v[3][b]);
    const double ab = sqrt(a.gama * pb / rhob);
    if (ub0 >= ab) {
      for (int v = 0; v < 4; ++v) q.v[v][b] = q.v[v][m1];
    } else {
      const double e = q.v[3][b];
      for (int t = 1; t <= 3; ++t) q.v[3][g2(g, -t, j)] = e;
    }
  }
  if (a.dir1) {
    for (int t = 0; t <= a.hx; ++t)
      for (int v = 0; v < 4; ++v) q.v[v][g2(g, g.n0 - 1 + t, j)] = a.f1[v];
  } else {
    for (int v = 0; v < 4; ++v) {  // outlet
      const double val = q.v[v][g2(g, g.n0 - 2, j)];
      for (int t = 0; t <= a.hx; ++t) q.v[v][g2(g, g.n0 - 1 + t, j)] = val;
    }
  }
}

// SymmetryBC (symmetry.py) of column i on an x1 face whose boundary row is jb, the interior on the
// side sg: the halo point jb - sg t mirrors jb + sg t with the normal momentum reversed; the boundary
// point keeps its values.
__device__ __forceinline__ void sym2_point(const Grid &g, const Q4 &q, int i, int jb, int sg, int t) {
  const int64_t h = g2(g, i, jb - sg * t), m = g2(g, i, jb + sg * t);
  q.v[0][h] = q.v[0][m];
  q.v[1][h] = q.v[1][m];
  q.v[2][h] = -q.v[2][m];
  q.v[3][h] = q.v[3][m];
}

// isothermal wall halo point -t of column i (t = 1 also sets the wall point itself and the
// Dirichlet top face of the column)
__device__ __forceinline__ void bc2_col(const Grid &g, const Q4 &q, const BC2Args &a, int i, int t) {
  if (a.adiy0) {  // adiabatic wall at x1 = 0 (halo point t), symmetry face at the top (with t = 1)
    auto at = [&](int j) { return g2(g, i, j); };
    adia2_line(q, a, at, 0, 1, t, t);  // t = 1 also sets the wall point
    if (t == 1)
      for (int u = 1; u <= a.hy; ++u) sym2_point(g, q, i, g.n1 - 1, -1, u);
    return;
  }
  if (a.sym0) {
    sym2_point(g, q, i, 0, 1, t);
    if (t == 1) {
      if (a.sym1) {
        for (int u = 1; u <= a.hy; ++u) sym2_point(g, q, i, g.n1 - 1, -1, u);
      } else {
        const double x0 = a.delta0 * i;  // Dirichlet top face
        for (int j = g.n1 - 1; j < g.n1 + a.hy; ++j)
          for (int v = 0; v < 4; ++v) q.v[v][g2(g, i, j)] = x0 > a.xs ? a.st.hi[v] : a.st.lo[v];
      }
    }
    return;
  }
  const double M2 = a.Minf * a.Minf, gama = a.gama;
  const int64_t w = g2(g, i, 0), a1 = g2(g, i, 1);
  // the wall point after this face: zero momentum, energy from Twall; its pressure
  // (gama-1) (rhoE - |rhou|^2 / (2 rho)) is exactly (gama-1) rhoE there
  const double rw = q.v[0][w], ew = a.Twall * (1.0 / M2) * rw / (gama * (gama - 1.0));
  const double Pw = (gama - 1) * ew;
  const double Ta = M2 * gama * (gama - 1) *
                    (-(0.5 * q.v[1][a1] * q.v[1][a1] + 0.5 * q.v[2][a1] * q.v[2][a1]) / q.v[0][a1] + q.v[3][a1]) /
                    q.v[0][a1];
  const int64_t m = g2(g, i, t), hh = g2(g, i, -t);
  const double um0 = q.v[1][m] / q.v[0][m], um1 = q.v[2][m] / q.v[0][m];
  const double Tt = (t + 1) * a.Twall - t * Ta;
  const double rh = M2 * gama * Pw / Tt;
  q.v[0][hh] = rh;
  q.v[1][hh] = -rh * um0;
  q.v[2][hh] = -rh * um1;
  q.v[3][hh] = (1.0 / (gama - 1)) * Pw + 0.5 * rh * (um0 * um0 + um1 * um1);
  if (a.wall1) {  // the channel's second wall: row n1-1, halo rows n1..n1+3 (t = 1..3 here, 4 with t = 1)
    const int jw = g.n1 - 1;
    const int64_t w1 = g2(g, i, jw), b1 = g2(g, i, jw - 1);
    const double ew1 = a.Twall * (1.0 / M2) * q.v[0][w1] / (gama * (gama - 1.0)), Pw1 = (gama - 1) * ew1;
    const double Tb = M2 * gama * (gama - 1) *
                      (-(0.5 * q.v[1][b1] * q.v[1][b1] + 0.5 * q.v[2][b1] * q.v[2][b1]) / q.v[0][b1] + q.v[3][b1]) /
                      q.v[0][b1];
    const int us[2] = {t, t == 1 ? 4 : 0};
    for (int k = 0; k < 2; ++k) {
      const int u = us[k];
      if (!u) continue;
      const int64_t m1 = g2(g, i, jw - u), h1 = g2(g, i, jw + u);
      const double v0 = q.v[1][m1] / q.v[0][m1], v1 = q.v[2][m1] / q.v[0][m1];
      const double Tu = (u + 1) * a.Twall - u * Tb, rh1 = M2 * gama * Pw1 / Tu;
      q.v[0][h1] = rh1;
      q.v[1][h1] = -rh1 * v0;
      q.v[2][h1] = -rh1 * v1;
      q.v[3][h1] = (1.0 / (gama - 1)) * Pw1 + 0.5 * rh1 * (v0 * v0 + v1 * v1);
    }
    if (t == 1) {
      q.v[1][w1] = 0.0;
      q.v[2][w1] = 0.0;
      q.v[3][w1] = ew1;
    }
  }
  if (t == 1) {
    q.v[1][w] = 0.0;
    q.v[2][w] = 0.0;
    q.v[3][w] = ew;
    if (a.wall1) return;
    const double x0 = a.delta0 * i;  // Dirichlet top face
    for (int j = g.n1 - 1; j < g.n1 + a.hy; ++j)
      for (int v = 0; v < 4; ++v) q.v[v][g2(g, i, j)] = x0 > a.xs ? a.st.hi[v] : a.st.lo[v];
  }
}

// The periodic exchange of axis d of a doubly periodic 2D block (exchange.py:9-57): the hx (hy) halo
// points of every padded row (column) take the interior points one period away.
__global__ void k2_wrap(Grid g, Q4 q, int d, int hx, int hy) {
  const int h = d == 0 ? hx : hy, len = d == 0 ? g.n1 + 2 * hy : g.n0 + 2 * hx, n = d == 0 ? g.n0 : g.n1;
  const int64_t N = (int64_t)4 * len * h;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / ((int64_t)len * h)), r = (int)(t % ((int64_t)len * h));
    const int a = r / h - (d == 0 ? hy : hx), k = r % h + 1;  // the row (column) and the halo depth
    double *f = q.v[v];
    if (d == 0) {
      f[g2(g, -k, a)] = f[g2(g, n - k, a)];
      f[g2(g, n - 1 + k, a)] = f[g2(g, k - 1, a)];
    } else {
      f[g2(g, a, -k)] = f[g2(g, a, n - k)];
      f[g2(g, a, n - 1 + k)] = f[g2(g, a, k - 1)];
    }
  }
}

// "Save equations" of the two-register RK3: qold (the context's RK register) = q on the interior
__global__ void k2_save(Grid g, Q4 q, Q4 qold, int nv) {
  const int64_t N = (int64_t)g.n0 * g.n1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = g2(g, (int)(t % g.n0), (int)(t / g.n0));
    for (int v = 0; v < nv; ++v) qold.v[v][c] = q.v[v][c];
  }
}

constexpr int BC2_THREADS = 128;
__global__ void __launch_bounds__(BC2_THREADS) k2_bc(Grid g, Q4 q, BC2Args a, int row_blocks) {
  const int tid = threadIdx.x;
  if (blockIdx.x == 0) {
    for (int j = -3 + tid; j < g.n1 + a.hy; j += BC2_THREADS)
      if (j <= 3 || j >= g.n1 - 5) bc2_row(g, q, a, j);
    __syncthreads();
    for (int w = tid; w < 3 * (g.n0 + a.hx + 3); w += BC2_THREADS) {
      const int i = w / 3 - 3;
      if (i <= 0 || i >= g.n0 - 2) bc2_col(g, q, a, i, w % 3 + 1);
    }
  } else if ((int)blockIdx.x <= row_blocks) {
    const int j = 4 + ((int)blockIdx.x - 1) * BC2_THREADS + tid;
    if (j < g.n1 - 5) bc2_row(g, q, a, j);
  } else {
    const int w = ((int)blockIdx.x - 1 - row_blocks) * BC2_THREADS + tid;
    const int i = 1 + w / 3;
    if (i < g.n0 - 2) bc2_col(g, q, a, i, w % 3 + 1);
  }
}

template <typename T> struct Q4T {
  T *v[4];
};

// FP64 master -> working state (mixed path), every padded point.
__global__ void k2_to_state(int64_t numel, Q4 src, Q4T<float> dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < numel; t += (int64_t)gridDim.x * blockDim.x)
    for (int v = 0; v < 4; ++v) dst.v[v][t] = cvt_f64_f32(src.v[v][t]);
}

// ---------------------------------------------------------------------------------------------
// constituent relations over -3..n+3 (u, p, a) with T and Sutherland mu
// ---------------------------------------------------------------------------------------------
template <typename T> struct Prims {
  T *u0, *u1, *p, *a, *T_, *mu;
};

// Over every padded point (-4 .. n+3) from the FP64 master state.  Mixed: the FP32 working state is
// written here (the FP64 -> FP32 rounding of the stage), and u, p, T come out rounded once from the
// FP32 values (prims_f32).  FP64: the master is the state.
template <typename T>
__global__ void k2_prims(Grid g, Q4 q64, Q4T<float> qs, Prims<T> pr, double gama, double Minf, double suth) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - 4, j = blockIdx.y * blockDim.y + threadIdx.y - 4;
  if (i >= g.n0 + 4 || j >= g.n1 + 4) return;
  const int64_t n = g2(g, i, j);
  T r, u0, u1, p, Tt, ir;
  const T gm = T(gama);
  if constexpr (sizeof(T) == 4) {
    float qv[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      qv[v] = cvt_f64_f32(q64.v[v][n]);
      qs.v[v][n] = qv[v];
    }
    const float gm1 = (float)(gama - 1.0), gm1_lo = (float)((gama - 1.0) - (double)gm1);
    float u[3], p_lo;
    r = qv[0];
    prims_f32(qv[0], qv[1], qv[2], 0.0f, qv[3], gm1, gm1_lo, ir, u, p, p_lo);
    u0 = u[0];
    u1 = u[1];
    Tt = scaled_ratio_f32((float)(Minf * Minf * gama), p, p_lo, r, ir);
  } else {
    r = q64.v[0][n];
    ir = T(1) / r;
    u0 = q64.v[1][n] * ir;
    u1 = q64.v[2][n] * ir;
    p = (gm - T(1)) * (q64.v[3][n] - T(0.5) * r * u0 * u0 - T(0.5) * r * u1 * u1);
    Tt = T(Minf * Minf * gama) * p * ir;
  }
  pr.u0[n] = u0;
  pr.u1[n] = u1;
  pr.p[n] = p;
  pr.a[n] = sqrt_t(gm * p * ir);
  const T S = T(suth);
  pr.T_[n] = Tt;
  pr.mu[n] = suth < 0.0 ? T(1) : (S + T(1)) * Tt * sqrt_t(Tt) / (S + Tt);  // suth < 0: constant mu = 1
}

// ---------------------------------------------------------------------------------------------
// adaptive TENO cut-off (schemes/spatial/teno.py:430-443) from the modified Ducros sensor
// (schemes/spatial/shock_sensors.py:12-49), one value per interface left point
// ---------------------------------------------------------------------------------------------
// 10^-k for k = 0..22, as decimal literals (the correctly rounded values pow(10, -k) returns)
__constant__ double c_p10n[23] = {1e0,   1e-1,  1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,
                                  1e-8,  1e-9,  1e-10, 1e-11, 1e-12, 1e-13, 1e-14, 1e-15,
                                  1e-16, 1e-17, 1e-18, 1e-19, 1e-20, 1e-21, 1e-22};

struct Sensor2Args {
  double inv_d0, inv_d1, a1, a2, eps;
  int clx, cly;  // Carpenter faces of x0 and x1 (d1c)
};

__device__ __forceinline__ float tanh_t(float x) { return tanhf(x); }
__device__ __forceinline__ double tanh_t(double x) { return tanh(x); }

// Over i in [-1, n0], j in [-1, n1] (every interface's left point along either axis).  On the
// interior, with the derivatives' one-sided closures and the x1 metric (d/dx1 = D11 d/dxi1):
//   theta = (1/2 - 1/2 tanh(2.5 + 250 div)) div^2 / (eps + div^2 + om^2),
//   div = du0/dx0 + du1/dx1, om = du1/dx0 - du0/dx1;
// theta = 0 on the other points (the sensor's range is the interior).  The cut-off is
// C_T = 10^-floor(a1 - a2 (1 - (1 - theta)^4 (1 + 4 theta))), formed in FP64 in both precisions.
template <typename T>
__global__ void k2_sensor_ct(Grid g, Prims<const T> pr, const double *D11, T *ct, Sensor2Args sa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - 1, j = blockIdx.y * blockDim.y + threadIdx.y - 1;
  if (i > g.n0 || j > g.n1) return;
  const int64_t n = g2(g, i, j);
  double th = 0.0;
  if (i >= 0 && i < g.n0 && j >= 0 && j < g.n1) {
    const int64_t sy = g.sy;
    auto U0x = [&](int o) { return pr.u0[n + o]; };
    auto U1x = [&](int o) { return pr.u1[n + o]; };
    auto U0y = [&](int o) { return pr.u0[n + o * sy]; };
    auto U1y = [&](int o) { return pr.u1[n + o * sy]; };
    const T id0 = T(sa.inv_d0), id1 = T(sa.inv_d1);
    const T l0 = id0 * d1c<T>(U0x, i, g.n0, sa.clx), l1 = id0 * d1c<T>(U1x, i, g.n0, sa.clx);
    const T l2 = id1 * d1c<T>(U0y, j, g.n1, sa.cly), l3 = id1 * d1c<T>(U1y, j, g.n1, sa.cly);
    const T D = T(D11[n]);
    const T div = l0 + l3 * D, om = l1 - l2 * D;
    const T sw = T(0.5) - T(0.5) * tanh_t(T(250) * l0 + T(250) * l3 * D + T(2.5));
    th = (double)(sw * (div * div) / (T(sa.eps) + div * div + om * om));
  }
  const double w = 1.0 - th;
  const double k = floor(sa.a1 - sa.a2 * (1.0 - (w * w) * (w * w) * (4.0 * th + 1.0)));
  const double c = (k >= 0.0 && k <= 22.0) ? c_p10n[(int)k] : pow(10.0, -k);
  ct[n] = T(c);
}

// ---------------------------------------------------------------------------------------------
// characteristic fluxes (4 conserved variables) with WENO5-JS or TENO5
// ---------------------------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T w5_side(T f0, T f1, T f2, T f3, T f4, T eps) {
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T t0 = f2 - T(2) * f3 + f4, s0 = T(3) * f2 - T(4) * f3 + f4;
  const T t1 = f1 - T(2) * f2 + f3, s1 = f1 - f3;
  const T t2 = f0 - T(2) * f1 + f2, s2 = f0 - T(4) * f1 + T(3) * f2;
  const T e0 = c13 * t0 * t0 + c14 * s0 * s0 + eps, e1 = c13 * t1 * t1 + c14 * s1 * s1 + eps,
          e2 = c13 * t2 * t2 + c14 * s2 * s2 + eps;
  const T a0 = T(3.0 / 10.0) * rcp2(e0 * e0), a1 = T(3.0 / 5.0) * rcp2(e1 * e1), a2 = T(1.0 / 10.0) * rcp2(e2 * e2);
  const T p0 = T(1.0 / 6.0) * f2 + T(5.0 / 12.0) * f3 - T(1.0 / 12.0) * f4;
  const T p1 = T(-1.0 / 12.0) * f1 + T(5.0 / 12.0) * f2 + T(1.0 / 6.0) * f3;
  const T p2 = T(1.0 / 6.0) * f0 - T(7.0 / 12.0) * f1 + T(11.0 / 12.0) * f2;
  return (a0 * p0 + a1 * p1 + a2 * p2) * rcp2(a0 + a1 + a2);
}

// TENO5 with a fixed cut-off (schemes/spatial/teno.py:57-213, 407-465) on f = CF +- lambda CS,
// ordered from the far upwind point to the far downwind one.  Smoothness indicators of the halved
// values; alpha_r = (1 + |b0 - b2| / (eps + b_r))^6 for the central (0), downwind (1) and upwind (2)
// candidates; delta_r = 0 where alpha_r / sum < C_T; weights d = (11/20, 2/5, 1/20).  The
// normalised weights are formed from the ratios m_r / max m so that (.)^6 cannot overflow.
template <typename T> __device__ __forceinline__ T t5_side(T f0, T f1, T f2, T f3, T f4, T eps, T ct) {
  const T h0 = T(0.5) * f0, h1 = T(0.5) * f1, h2 = T(0.5) * f2, h3 = T(0.5) * f3, h4 = T(0.5) * f4;
  const T c13 = T(13.0 / 12.0), c14 = T(0.25);
  const T x0 = h1 - h3, y0 = h1 - T(2) * h2 + h3;
  const T x1 = h2 - T(2) * h3 + h4, y1 = T(3) * h2 - T(4) * h3 + h4;
  const T x2 = h0 - T(4) * h1 + T(3) * h2, y2 = h0 - T(2) * h1 + h2;
  const T b0 = c14 * x0 * x0 + c13 * y0 * y0;
  const T b1 = c13 * x1 * x1 + c14 * y1 * y1;
  const T b2 = c14 * x2 * x2 + c13 * y2 * y2;
  const T tau = abs_t(b0 - b2);
  const T m0 = T(1) + tau / (eps + b0), m1 = T(1) + tau / (eps + b1), m2 = T(1) + tau / (eps + b2);
  const T mm = max_t(m0, max_t(m1, m2));
  const T n0 = m0 / mm, n1 = m1 / mm, n2 = m2 / mm;
  const T q0 = (n0 * n0) * (n0 * n0) * (n0 * n0), q1 = (n1 * n1) * (n1 * n1) * (n1 * n1),
          q2 = (n2 * n2) * (n2 * n2) * (n2 * n2);
  const T iq = T(1) / (q0 + q1 + q2);
  const T d0 = ct > q0 * iq ? T(0) : T(1), d1 = ct > q1 * iq ? T(0) : T(1), d2 = ct > q2 * iq ? T(0) : T(1);
  const T w0 = T(0.55) * d0, w1 = T(0.4) * d1, w2 = T(0.05) * d2;
  const T iw = T(1) / (w0 + w1 + w2);
  return (w0 * (T(-1.0 / 12.0) * f1 + T(5.0 / 12.0) * f2 + T(1.0 / 6.0) * f3) +
          w1 * (T(1.0 / 6.0) * f2 + T(5.0 / 12.0) * f3 - T(1.0 / 12.0) * f4) +
          w2 * (T(1.0 / 6.0) * f0 - T(7.0 / 12.0) * f1 + T(11.0 / 12.0) * f2)) *
         iw;
}

enum { S2_RHO = 0, S2_RU0, S2_RU1, S2_E, S2_P, S2_A, S2_UD, S2_NF };
// FP32 tiles also stage each point's double-float flux (hi, lo of 4 components)
enum { S2_FH = S2_NF, S2_FL = S2_NF + 4 };
template <typename T> __host__ __device__ constexpr int s2nf() { return sizeof(T) == 4 ? S2_NF + 8 : S2_NF; }

template <typename T> struct W2 {
  T Q[4], ud, a, p;
};

// FP32 flux of one point along D, (Q_{1+D}, Q_{1+c} u_D + delta_cD p, (Q_3 + p) u_D), as a double-float
// sum h + l: u_D and p come with their remainders (the division residual of u_D is exact, prims_f32
// gives p_lo), products split by FMA, sums by two-sum.  The characteristic projections below act on
// differences of these fluxes between nearby points, which FP32 rounding of the O(1) flux itself
// would swamp.
template <int D>
__device__ __forceinline__ void point_flux2_ff(float rho, float m0, float m1, float E, float gm1, float gm1_lo,
                                               float h[4], float l[4]) {
  float ir, u[3], p, p_lo;
  prims_f32(rho, m0, m1, 0.0f, E, gm1, gm1_lo, ir, u, p, p_lo);
  const float m[2] = {m0, m1};
  const float ud = u[D], ud_lo = fmaf(-ud, rho, m[D]) * ir;
  h[0] = m[D];
  l[0] = 0.0f;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const float ph = __fmul_rn(m[c], ud);
    const float pl = fmaf(m[c], ud, -ph) + m[c] * ud_lo;
    if (c == D) {
      const float sh = __fadd_rn(ph, p), bv = __fsub_rn(sh, ph);
      const float es = __fadd_rn(__fsub_rn(ph, __fsub_rn(sh, bv)), __fsub_rn(p, bv));
      h[1 + c] = sh;
      l[1 + c] = es + pl + p_lo;
    } else {
      h[1 + c] = ph;
      l[1 + c] = pl;
    }
  }
  const float sh = __fadd_rn(E, p), bv = __fsub_rn(sh, E);
  const float es = __fadd_rn(__fsub_rn(E, __fsub_rn(sh, bv)), __fsub_rn(p, bv));
  const float hh = __fmul_rn(sh, ud);
  h[3] = hh;
  l[3] = fmaf(sh, ud, -hh) + fmaf(es + p_lo, ud, sh * ud_lo);
}

// Both sides of one characteristic reconstruction (fp: CF + lambda CS, fm: CF - lambda CS at the six
// window points): TENO5 (t5_side), WENO5-JS (w5_side), WENO5-Z (weno5_side, weno.py:283-331) or TENO6
// (teno6_side, teno.py:94-192, 216-234, six points per side).
template <typename T, int SCH>
__device__ __forceinline__ T recon2(const T (&fp)[6], const T (&fm)[6], T eps, T ct) {
  if constexpr (SCH == SCH_TENO)
    return t5_side(fp[0], fp[1], fp[2], fp[3], fp[4], eps, ct) + t5_side(fm[5], fm[4], fm[3], fm[2], fm[1], eps, ct);
  else if constexpr (SCH == SCH_TENO6)
    return teno6_side<T>(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], true, eps, ct) +
           teno6_side<T>(fm[5], fm[4], fm[3], fm[2], fm[1], fm[0], false, eps, ct);
  else if constexpr (SCH == SCH_Z)
    return weno5_side<T, SCH_Z>(fp[0], fp[1], fp[2], fp[3], fp[4], eps) +
           weno5_side<T, SCH_Z>(fm[5], fm[4], fm[3], fm[2], fm[1], eps);
  else
    return w5_side(fp[0], fp[1], fp[2], fp[3], fp[4], eps) + w5_side(fm[5], fm[4], fm[3], fm[2], fm[1], eps);
}

// The state of the characteristic system at the interface between the points l and r (conserved
// ql, qr, pressures and sound speeds): RoeAverage (averaging.py:62-114; rho = sqrt(rho_l rho_r), u
// and H weighted by sqrt(rho), a from H) or, with simple, SimpleAverage (averaging.py:31-59: the
// arithmetic means of rho, u = rhou/rho and a).
template <typename T>
__device__ __forceinline__ void avg2(const T (&ql)[4], const T (&qr)[4], T pl, T pr, T al, T ar, T gm1, bool simple,
                                     T &rho, T (&u)[2], T &a) {
  const T rl = ql[0], rr = qr[0];
  if (simple) {
    rho = T(0.5) * (rl + rr);
#pragma unroll
    for (int c = 0; c < 2; ++c) u[c] = T(0.5) * (qr[1 + c] / rr + ql[1 + c] / rl);
    a = T(0.5) * (al + ar);
    return;
  }
  const T sl = sqrt_t(rl), sr = sqrt_t(rr);
  rho = sqrt_t(rl * rr);
  const T inv_s = T(1) / (sl + sr);
#pragma unroll
  for (int c = 0; c < 2; ++c) u[c] = inv_s * (sl * (ql[1 + c] / rl) + sr * (qr[1 + c] / rr));
  const T Hh = inv_s * ((pl + ql[3]) / sl + (pr + qr[3]) / sr);
  a = sqrt_t(gm1 * (Hh - T(0.5) * (u[0] * u[0] + u[1] * u[1])));
}

// Characteristic flux between window points 2 and 3 along D (2D Euler eigensystem for a unit
// normal, physical_models/euler_eigensystem.py:77-105; the block's metric is diagonal so the
// eigensystem is Cartesian).  Dense rows share g = phi X0 - (g-1) u.X + (g-1) X3, h = X_{1+D} - u_D X0.
template <typename T, int D, int SCH>
__device__ __forceinline__ void flux2(const W2<T> (&W)[6], T gama, T eps, T ct, T out[4], bool simple) {
  constexpr int E = 1 - D;
  const T s = D == 0 ? T(1) : T(-1);
  const T gm1 = gama - T(1);
  const T rl = W[2].Q[0], rr = W[3].Q[0];
  T rho, u[2], a;
  avg2(W[2].Q, W[3].Q, W[2].p, W[3].p, W[2].a, W[3].a, gm1, simple, rho, u, a);
  const T usq = u[0] * u[0] + u[1] * u[1];
  const T ia = T(1) / a, irho = T(1) / rho;
  const T phi = gm1 * T(0.5) * usq;
  const T bt = T(0.70710678118654752440) * irho * ia, al = T(0.70710678118654752440) * rho * ia;
  const T ia2 = ia * ia, btA = bt * a;
  T lu = T(0), lp = T(0), lm = T(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    lu = max_t(lu, abs_t(W[t].ud));
    lp = max_t(lp, abs_t(W[t].ud + W[t].a));
    lm = max_t(lm, abs_t(W[t].a - W[t].ud));
  }
  auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    return recon2<T, SCH>(fp, fm, eps, ct);
  };
  T r0, r1, r2, r3;
  {
    T cf[6], cs[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {  // shear row: (s/rho)(u_E X0 - X_{1+E})
      cf[t] = s * irho * (u[E] * W[t].Q[1 + D] - W[t].Q[1 + E] * W[t].ud);
      cs[t] = s * irho * (u[E] * W[t].Q[0] - W[t].Q[1 + E]);
    }
    r1 = recon(cf, cs, lu);
    T gQ[6], gF[6], hQ[6], hF[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const W2<T> &w = W[t];
      const T dq = u[0] * w.Q[1] + u[1] * w.Q[2];
      gQ[t] = phi * w.Q[0] - gm1 * dq + gm1 * w.Q[3];
      hQ[t] = w.Q[1 + D] - u[D] * w.Q[0];
      gF[t] = phi * w.Q[1 + D] - gm1 * (w.ud * dq + u[D] * w.p) + gm1 * (w.p + w.Q[3]) * w.ud;
      hF[t] = w.Q[1 + D] * w.ud + w.p - u[D] * w.Q[1 + D];
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = W[t].Q[1 + D] - gF[t] * ia2;
      cs[t] = W[t].Q[0] - gQ[t] * ia2;
    }
    r0 = recon(cf, cs, lu);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] + btA * hF[t];
      cs[t] = bt * gQ[t] + btA * hQ[t];
    }
    r2 = recon(cf, cs, lp);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] - btA * hF[t];
      cs[t] = bt * gQ[t] - btA * hQ[t];
    }
    r3 = recon(cf, cs, lm);
  }
  const T sac = r2 + r3, dac = r2 - r3;
  const T hh = (phi + a * a) / gm1;
  out[0] = r0 + al * sac;
#pragma unroll
  for (int c = 0; c < 2; ++c) out[1 + c] = u[c] * r0 + al * (u[c] * sac + (c == D ? a * dac : T(0)));
  out[3] = (phi / gm1) * r0 + al * (hh * sac + u[D] * a * dac);
  out[1 + E] -= s * rho * r1;
  out[3] -= s * rho * u[E] * r1;
}

// FP32: the same characteristic flux in difference form about window point 2 (point i): the
// reconstructions reproduce constants (WENO and TENO candidates are consistent, the weights sum to
// one) and the splitting is linear, so projecting Q_t - Q_i and F_t - F_i gives LEV.(F^ - F_i) and
// REV maps it to G = F_{i+1/2} - F_i.  dF[t][v] = F_t - F_i from the double-float point fluxes.
// Returns G; the caller differences (F_i - F_{i-1}) + (G_i - G_{i-1}).
// T = double: the same flux in FP64 arithmetic on the window's FP32 values (next to strong shocks),
// rounded to FP32 once.
template <typename T, int D, int SCH>
__device__ __forceinline__ void flux2_delta(const W2<float> (&W)[6], const float (&dFf)[6][4], T gama, T eps, T ct,
                                            float out[4], bool simple) {
  T dF[6][4];
#pragma unroll
  for (int t = 0; t < 6; ++t)
#pragma unroll
    for (int v = 0; v < 4; ++v) dF[t][v] = T(dFf[t][v]);
  constexpr int E = 1 - D;
  const T s = D == 0 ? T(1) : T(-1);
  const T gm1 = gama - T(1);
  T rho, u[2], a;
  {
    const T ql[4] = {T(W[2].Q[0]), T(W[2].Q[1]), T(W[2].Q[2]), T(W[2].Q[3])};
    const T qr[4] = {T(W[3].Q[0]), T(W[3].Q[1]), T(W[3].Q[2]), T(W[3].Q[3])};
    avg2(ql, qr, T(W[2].p), T(W[3].p), T(W[2].a), T(W[3].a), gm1, simple, rho, u, a);
  }
  const T usq = u[0] * u[0] + u[1] * u[1];
  const T ia = T(1) / a, irho = T(1) / rho;
  const T phi = gm1 * T(0.5) * usq;
  const T bt = T(0.70710678118654752440) * irho * ia, al = T(0.70710678118654752440) * rho * ia;
  const T ia2 = ia * ia, btA = bt * a;
  T lu = T(0), lp = T(0), lm = T(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    lu = max_t(lu, abs_t(T(W[t].ud)));
    lp = max_t(lp, abs_t(T(W[t].ud) + T(W[t].a)));
    lm = max_t(lm, abs_t(T(W[t].a) - T(W[t].ud)));
  }
  auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    return recon2<T, SCH>(fp, fm, eps, ct);
  };
  auto dQ = [&](int t, int v) -> T { return t == 2 ? T(0) : T(W[t].Q[v]) - T(W[2].Q[v]); };
  T r0, r1, r2, r3;
  {
    T cf[6], cs[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {  // shear row: (s/rho)(u_E X0 - X_{1+E})
      cf[t] = s * irho * (u[E] * dF[t][0] - dF[t][1 + E]);
      cs[t] = s * irho * (u[E] * dQ(t, 0) - dQ(t, 1 + E));
    }
    r1 = recon(cf, cs, lu);
    T gQ[6], gF[6], hQ[6], hF[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      gQ[t] = phi * dQ(t, 0) - gm1 * (u[0] * dQ(t, 1) + u[1] * dQ(t, 2)) + gm1 * dQ(t, 3);
      hQ[t] = dQ(t, 1 + D) - u[D] * dQ(t, 0);
      gF[t] = phi * dF[t][0] - gm1 * (u[0] * dF[t][1] + u[1] * dF[t][2]) + gm1 * dF[t][3];
      hF[t] = dF[t][1 + D] - u[D] * dF[t][0];
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = dF[t][0] - gF[t] * ia2;
      cs[t] = dQ(t, 0) - gQ[t] * ia2;
    }
    r0 = recon(cf, cs, lu);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] + btA * hF[t];
      cs[t] = bt * gQ[t] + btA * hQ[t];
    }
    r2 = recon(cf, cs, lp);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] - btA * hF[t];
      cs[t] = bt * gQ[t] - btA * hQ[t];
    }
    r3 = recon(cf, cs, lm);
  }
  const T sac = r2 + r3, dac = r2 - r3;
  const T hh = (phi + a * a) / gm1;
  T G[4];
  G[0] = r0 + al * sac;
#pragma unroll
  for (int c = 0; c < 2; ++c) G[1 + c] = u[c] * r0 + al * (u[c] * sac + (c == D ? a * dac : T(0)));
  G[3] = (phi / gm1) * r0 + al * (hh * sac + u[D] * a * dac);
  G[1 + E] -= s * rho * r1;
  G[3] -= s * rho * u[E] * r1;
#pragma unroll
  for (int v = 0; v < 4; ++v) out[v] = float(G[v]);
}

template <int D> struct T2Tile;
template <> struct T2Tile<0> { static constexpr int TI = 64, TA = 4; };
template <> struct T2Tile<1> { static constexpr int TI = 24, TA = 16; };  // static smem < 48 KB in FP64

// Interface fluxes along D for a tile and the flux difference -(F_i - F_{i-1})/delta (times D11 for
// x1), written into this direction's residual array.  TENO's cut-off is ct_d, or with ctp set the
// per-point value at the interface's left point.
// SH (FP32 only): interfaces next to strong shocks (pressure ratio of points i, i+1 above `shock`)
// form their flux in FP64 arithmetic; a separate instantiation, since the FP64 path raises the
// kernel's registers from ~94 to ~160 and halves the resident blocks.
template <typename T, int D, int SCH, bool SH = false>
__global__ void __launch_bounds__(256) k2_flux(Grid g, Q4T<const T> q, Prims<const T> pr, const double *D11,
                                               Q4T<T> res, double gama_d, double eps_d, double ct_d, double inv_dd,
                                               const T *ctp, double shock, int simple) {
  using Tl = T2Tile<D>;
  constexpr int TI = Tl::TI, TA = Tl::TA, NPT = TI + 5;
  constexpr int NF = s2nf<T>();
  __shared__ T sf[NF][NPT][TA];
  __shared__ T sfl[4][TI][TA];
  __shared__ T sdf[sizeof(T) == 4 ? 4 : 1][TI][TA];  // FP32: F(left point) - F(the point before)
  const int tid = threadIdx.x;
  const int nd = D == 0 ? g.n0 : g.n1, na = D == 0 ? g.n1 : g.n0;
  const int d0 = (D == 0 ? blockIdx.x : blockIdx.y) * (TI - 1);
  const int a0 = (D == 0 ? blockIdx.y : blockIdx.x) * TA;
  auto coord = [&](int c, int a, int &i, int &j) {
    if (D == 0) { i = c; j = a0 + a; }
    else { i = a0 + a; j = c; }
  };
  for (int t = tid; t < NPT * TA; t += 256) {
    int pos, a;
    if (D == 0) { a = t / NPT; pos = t % NPT; }
    else { pos = t / TA; a = t % TA; }
    const int c = d0 - 3 + pos;
    if (c > nd + 2 || a0 + a >= na) continue;
    int i, j;
    coord(c, a, i, j);
    const int64_t m = g2(g, i, j);
    sf[S2_RHO][pos][a] = q.v[0][m];
    sf[S2_RU0][pos][a] = q.v[1][m];
    sf[S2_RU1][pos][a] = q.v[2][m];
    sf[S2_E][pos][a] = q.v[3][m];
    sf[S2_P][pos][a] = pr.p[m];
    sf[S2_A][pos][a] = pr.a[m];
    sf[S2_UD][pos][a] = D == 0 ? pr.u0[m] : pr.u1[m];
    if constexpr (sizeof(T) == 4) {
      const float gm1 = (float)(gama_d - 1.0), gm1_lo = (float)((gama_d - 1.0) - (double)gm1);
      float h[4], l[4];
      point_flux2_ff<D>(q.v[0][m], q.v[1][m], q.v[2][m], q.v[3][m], gm1, gm1_lo, h, l);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        sf[S2_FH + v][pos][a] = h[v];
        sf[S2_FL + v][pos][a] = l[v];
      }
    }
  }
  __syncthreads();
  const T gama = T(gama_d), eps = T(eps_d), ct = T(ct_d);
  for (int t = tid; t < TI * TA; t += 256) {
    int m, a;
    if (D == 0) { a = t / TI; m = t % TI; }
    else { m = t / TA; a = t % TA; }
    if (d0 - 1 + m > nd - 1 || a0 + a >= na) continue;
    W2<T> W[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      W[k].Q[0] = sf[S2_RHO][m + k][a];
      W[k].Q[1] = sf[S2_RU0][m + k][a];
      W[k].Q[2] = sf[S2_RU1][m + k][a];
      W[k].Q[3] = sf[S2_E][m + k][a];
      W[k].p = sf[S2_P][m + k][a];
      W[k].a = sf[S2_A][m + k][a];
      W[k].ud = sf[S2_UD][m + k][a];
    }
    T ctl = ct;
    if (SCH == SCH_TENO && ctp) {
      int i, j;
      coord(d0 - 1 + m, a, i, j);
      ctl = ctp[g2(g, i, j)];
    }
    T fl[4];
    if constexpr (sizeof(T) == 4) {
      // F_t - F_i of the window from the staged double-float fluxes, each rounded once
      float dF[6][4];
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int v = 0; v < 4; ++v)
          dF[k][v] = k == 2 ? 0.0f
                            : __fsub_rn(sf[S2_FH + v][m + k][a], sf[S2_FH + v][m + 2][a]) +
                                  __fsub_rn(sf[S2_FL + v][m + k][a], sf[S2_FL + v][m + 2][a]);
      bool fp64 = false;
      if constexpr (SH) {
        const float pl = W[2].p, pr = W[3].p;
        fp64 = fmaxf(pl, pr) > (float)shock * fminf(pl, pr);
      }
      if (fp64) {
        if constexpr (SH) flux2_delta<double, D, SCH>(W, dF, gama_d, eps_d, ctp ? (double)ctl : ct_d, fl, simple);
      } else {
        flux2_delta<float, D, SCH>(W, dF, gama, eps, ctl, fl, simple);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) sdf[v][m][a] = -dF[1][v];  // F(point i) - F(point i-1)
    } else {
      flux2<T, D, SCH>(W, gama, eps, ctl, fl, simple);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) sfl[v][m][a] = fl[v];
  }
  __syncthreads();
  for (int t = tid; t < (TI - 1) * TA; t += 256) {
    int m, a;
    if (D == 0) { a = t / (TI - 1); m = t % (TI - 1); }
    else { m = t / TA; a = t % TA; }
    const int c = d0 + m;
    if (c >= nd || a0 + a >= na) continue;
    int i, j;
    coord(c, a, i, j);
    const int64_t gi = g2(g, i, j);
    // 1/delta (times D11 along x1) formed in FP64 and carried as an FP32 pair in mixed precision: one
    // rounding of it would scale every flux difference of the point the same way, step after step
    const double sc = D == 0 ? inv_dd : inv_dd * D11[gi];
    const T sc_hi = T(sc), sc_lo = T(sc - (double)sc_hi);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      T diff = sfl[v][m + 1][a] - sfl[v][m][a];
      if constexpr (sizeof(T) == 4) diff = sdf[v][m + 1][a] + diff;  // (F_i - F_{i-1}) + (G_i - G_{i-1})
      res.v[v][gi] = -mul_hl(diff, sc_hi, sc_lo);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// viscous terms (stretched metric, closures) + LS-RK3 update
// ---------------------------------------------------------------------------------------------
struct Visc2Args {
  double Re, kappa, inv_d0, inv_d1, inv_d2;
  int clx, cly;  // Carpenter faces of x0 and x1 (d1c)
};

// Central skew-symmetric convective terms of a Cartesian 2D block (laminar_channel.py's Skew(...), the
// form of the Taylor-Green script, parsing.py:75-111) with the faces' derivative closures:
//   R_rho = -sum_d skew(rho, d), R_rhou_i = -sum_d skew(rhou_i, d) - dp/dx_i,
//   R_rhoE = -sum_d skew(rhoE, d) - sum_d d(p u_d)/dx_d,  skew(phi, d) = (d(phi u_d) + u_d dphi + phi du_d)/2.
// A 32 x 8 tile stages rho, rhou0, rhou1, rhoE, u0, u1 and p with a 5-point margin in shared memory.
struct Skew2Args {
  double inv_d0, inv_d1;
  int clx, cly;
};

template <typename T>
__global__ void __launch_bounds__(256) k2_skew(Grid g, Q4T<const T> q, const T *u0, const T *u1, const T *pr, Q4T<T> r,
                                               Skew2Args sa) {
  constexpr int TX = 32, TY = 8, HM = 5, SX = TX + 2 * HM, SY = TY + 2 * HM;
  __shared__ T sm[7][SY][SX];  // rho rhou0 rhou1 rhoE u0 u1 p
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, tid = threadIdx.y * TX + threadIdx.x;
  for (int t = tid; t < SX * SY; t += TX * TY) {
    const int li = t % SX, lj = t / SX, gi = i0 - HM + li, gj = j0 - HM + lj;
    if (gi < -4 || gi >= g.n0 + 4 || gj < -4 || gj >= g.n1 + 4) continue;
    const int64_t m = g2(g, gi, gj);
#pragma unroll
    for (int v = 0; v < 4; ++v) sm[v][lj][li] = q.v[v][m];
    sm[4][lj][li] = u0[m];
    sm[5][lj][li] = u1[m];
    sm[6][lj][li] = pr[m];
  }
  __syncthreads();
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i >= g.n0 || j >= g.n1) return;
  const int li = threadIdx.x + HM, lj = threadIdx.y + HM;
  auto D = [&](int d, auto &&F) {  // first derivative along d of F(offset) at the point
    return d == 0 ? T(sa.inv_d0) * d1c<T>([&](int o) { return F(0, o); }, i, g.n0, sa.clx)
                  : T(sa.inv_d1) * d1c<T>([&](int o) { return F(1, o); }, j, g.n1, sa.cly);
  };
  auto at = [&](int f, int d, int o) -> T { return d == 0 ? sm[f][lj][li + o] : sm[f][lj + o][li]; };
  T R[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    T acc = T(0);
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const T dprod = D(d, [&](int dd, int o) { return at(v, dd, o) * at(4 + dd, dd, o); });
      const T dphi = D(d, [&](int dd, int o) { return at(v, dd, o); });
      const T du = D(d, [&](int dd, int o) { return at(4 + dd, dd, o); });
      acc += T(0.5) * (dprod + sm[4 + d][lj][li] * dphi + sm[v][lj][li] * du);
    }
    R[v] = -acc;
  }
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    R[1 + d] -= D(d, [&](int dd, int o) { return at(6, dd, o); });
    R[3] -= D(d, [&](int dd, int o) { return at(6, dd, o) * at(4 + dd, dd, o); });
  }
  const int64_t c = g2(g, i, j);
#pragma unroll
  for (int v = 0; v < 4; ++v) r.v[v][c] = R[v];
}

template <typename T> struct Q3T {
  T *v[3];
};

// Viscous terms of the momentum and energy equations at every interior point (the reference's
// "Viscous" kernels: Newtonian stress and Fourier heat flux with Sutherland mu, d/dx1 = D11 d/dxi1 and
// d2/dx1^2 = D11^2 d2/dxi1^2 + D11 SD111 d/dxi1, one-sided closures at the faces), into rv (momentum
// 0, momentum 1, energy).  A 32 x 8 tile stages u0, u1, T and mu of its points and of the V2H points
// around them in shared memory: the widest stencil, a one-sided closure or the nested x0/x1
// derivative, reaches V2H = 5 points.  Points outside the padded arrays are neither staged nor read.
constexpr int V2X = 32, V2Y = 8, V2H = 5;
template <typename T>
__global__ void __launch_bounds__(V2X * V2Y, 2) k2_visc(Grid g, Prims<const T> pr, const double *D11,
                                                        const double *SD111, Q3T<T> rv, Visc2Args va, int hx,
                                                        int hy) {
  constexpr int SX = V2X + 2 * V2H, SY = V2Y + 2 * V2H;
  __shared__ T sm[4][SY][SX];  // u0, u1, T, mu
  const int i0 = blockIdx.x * V2X, j0 = blockIdx.y * V2Y;
  const int tid = threadIdx.y * V2X + threadIdx.x;
  const T *src[4] = {pr.u0, pr.u1, pr.T_, pr.mu};
  for (int t = tid; t < SX * SY; t += V2X * V2Y) {
    const int li = t % SX, lj = t / SX;
    const int gi = i0 - V2H + li, gj = j0 - V2H + lj;
    if (gi < -hx || gi >= g.n0 + hx || gj < -hy || gj >= g.n1 + hy) continue;
    const int64_t m = g2(g, gi, gj);
#pragma unroll
    for (int f = 0; f < 4; ++f) sm[f][lj][li] = src[f][m];
  }
  __syncthreads();
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  if (i >= g.n0 || j >= g.n1) return;
  const int li = threadIdx.x + V2H, lj = threadIdx.y + V2H;
  const int64_t c = g2(g, i, j);
  const T id0 = T(va.inv_d0), id1 = T(va.inv_d1), iRe = T(1.0 / va.Re);
  const T Dm = T(D11[c]), S = T(SD111[c]), mu = sm[3][lj][li];
  T gr[2][2], h[2][2][2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    auto X = [&](int o) { return sm[k][lj][li + o]; };
    auto Y = [&](int o) { return sm[k][lj + o][li]; };
    gr[k][0] = id0 * d1c<T>(X, i, g.n0, va.clx);
    const T fy = id1 * d1c<T>(Y, j, g.n1, va.cly);
    gr[k][1] = Dm * fy;
    h[k][0][0] = id0 * id0 * d2c<T>(X, i, g.n0, va.clx);
    h[k][1][1] = Dm * Dm * (id1 * id1 * d2c<T>(Y, j, g.n1, va.cly)) + Dm * S * fy;
    // d/dx0 of the row j+o, then d/dxi1 of that column (inner axis x0 over the extended x1 range)
    auto inner = [&](int o) {
      return id0 * d1c<T>([&](int p) { return sm[k][lj + o][li + p]; }, i, g.n0, va.clx);
    };
    h[k][0][1] = h[k][1][0] = Dm * (id1 * d1c<T>(inner, j, g.n1, va.cly));
  }
  auto XT = [&](int o) { return sm[2][lj][li + o]; };
  auto YT = [&](int o) { return sm[2][lj + o][li]; };
  auto Xmu = [&](int o) { return sm[3][lj][li + o]; };
  auto Ymu = [&](int o) { return sm[3][lj + o][li]; };
  const T mux = id0 * d1c<T>(Xmu, i, g.n0, va.clx);
  const T muy = Dm * id1 * d1c<T>(Ymu, j, g.n1, va.cly);
  const T Tx = id0 * d1c<T>(XT, i, g.n0, va.clx);
  const T Tyx = id1 * d1c<T>(YT, j, g.n1, va.cly);
  const T Ty = Dm * Tyx;
  const T Txx = id0 * id0 * d2c<T>(XT, i, g.n0, va.clx);
  const T Tyy = Dm * Dm * (id1 * id1 * d2c<T>(YT, j, g.n1, va.cly)) + Dm * S * Tyx;
  const T div = gr[0][0] + gr[1][1];
  const T mug[2] = {mux, muy};
  const T uu[2] = {sm[0][lj][li], sm[1][lj][li]};
  T e = T(va.kappa) * (mu * (Txx + Tyy) + mux * Tx + muy * Ty);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    T v = T(0);
#pragma unroll
    for (int b = 0; b < 2; ++b) v += mug[b] * (gr[a][b] + gr[b][a] - (a == b ? T(2.0 / 3.0) * div : T(0))) * iRe;
    const T lap = h[a][0][0] + h[a][1][1];
    const T ddiv = h[0][a][0] + h[1][a][1];
    v += mu * iRe * (lap + ddiv * T(1.0 / 3.0));
    rv.v[a][c] = v;
    e += uu[a] * v;
#pragma unroll
    for (int b = 0; b < 2; ++b) e += mu * iRe * (gr[a][b] + gr[b][a] - (a == b ? T(2.0 / 3.0) * div : T(0))) * gr[a][b];
  }
  rv.v[2][c] = e;
}

// R = (x fluxes + x1 fluxes) + viscous terms at every interior point, then the LS-RK3 update
// du = dt R + A du, q += B du in FP64 (update = 1), or R itself into du (update = 0: osb_residual).
template <typename T>
__global__ void k2_rk(Grid g, Q4T<const T> rx, Q4T<const T> ry, Q3T<const T> rv, Q4 du, Q4 q64, double dt, double A,
                      double B, int update, int rk2, double f0, double f1) {
  const int64_t N = (int64_t)g.n0 * g.n1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)(t / g.n0);
    const int64_t c = g2(g, i, j);
    T R[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) R[v] = ry.v[0] ? rx.v[v][c] + ry.v[v][c] : rx.v[v][c];  // ry: x1 fluxes
    if (rv.v[0]) {  // viscous terms (none on Euler blocks)
      R[1] += rv.v[0][c];
      R[2] += rv.v[1][c];
      R[3] += rv.v[2][c];
    }
    if (f0 != 0.0 || f1 != 0.0) {  // the channel's forcing c_j (laminar_channel.py): -c_i, -c_j u_j
      const double ir = 1.0 / q64.v[0][c];
      R[1] -= T(f0);
      R[2] -= T(f1);
      R[3] -= T(f0 * (q64.v[1][c] * ir) + f1 * (q64.v[2][c] * ir));
    }
    if (update && rk2) {  // RungeKutta(3), two registers (rk_sbli.py:117-124): du holds qold
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double r = to_f64(R[v]), old = du.v[v][c];
        q64.v[v][c] = dt * B * r + old;
        du.v[v][c] = dt * A * r + old;
      }
    } else if (update) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double d = dt * to_f64(R[v]) + A * du.v[v][c];
        du.v[v][c] = d;
        q64.v[v][c] = B * d + q64.v[v][c];
      }
    } else {
#pragma unroll
      for (int v = 0; v < 4; ++v) du.v[v][c] = to_f64(R[v]);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------------------
static Q4 q4(double *const *a) {
  Q4 r;
  for (int v = 0; v < 4; ++v) r.v[v] = a[v];
  return r;
}
template <typename T> static Q4T<T> q4t(void *const *a) {
  Q4T<T> r;
  for (int v = 0; v < 4; ++v) r.v[v] = static_cast<T *>(a[v]);
  return r;
}

// the Carpenter faces of one axis as d1c's bit mask
static int closure_bits(const osb_plan_desc &p, int axis) {
  if (p.bc[axis][0] == OSB_BC_PERIODIC) return 4;
  return (p.closure[axis][0] == OSB_CLOSURE_CARPENTER ? 1 : 0) | (p.closure[axis][1] == OSB_CLOSURE_CARPENTER ? 2 : 0) |
         (p.closure[axis][0] == OSB_CLOSURE_NONE ? 8 : 0) | (p.closure[axis][1] == OSB_CLOSURE_NONE ? 16 : 0);
}

// The Carpenter first-derivative closure (Carpenter_scheme.py:90-102): weights = A^-1 B with the 4x4
// block A and the 4x6 block B of the published boundary operator, free parameters R1 and R2 as the
// reference sets them; solved once on the host (Gauss-Jordan, partial pivoting) and uploaded to the
// constant tables c_carp_d / c_carp_f (the same values for every context).
cudaError_t upload2_closure_weights() {
  const double R1 = -(2177.0 * std::sqrt(295369.0) - 1166427.0) / 25488.0;
  const double R2 = (66195.0 * std::sqrt(53.0) * std::sqrt(5573.0) - 35909375.0) / 101952.0;
  const double a = 216.0 * R2 + 2160.0 * R1, b = 81.0 * R2 + 675.0 * R1, e = 864.0 * R2 + 6480.0 * R1;
  const double f = 72.0 * R2 + 720.0 * R1, h = 108.0 * R2 + 756.0 * R1, u = 4104.0 * R2 + 32400.0 * R1;
  const double w = 1836.0 * R2 + 14580.0 * R1, y = 216.0 * R2 + 1620.0 * R1, z = 108.0 * R2 + 810.0 * R1;
  double M[4][10] = {
      {-(a - 2125.0) / 12960.0, (b + 415.0) / 540.0, -(f + 445.0) / 1440.0, -(h + 421.0) / 1296.0,
       -0.5, -(e + 305.0) / 4320.0, (y + 725.0) / 540.0, -(e + 3335.0) / 4320.0, 0.0, 0.0},
      {(b + 415.0) / 540.0, -(u + 11225.0) / 4320.0, (w + 7295.0) / 2160.0, -(a + 655.0) / 4320.0,
       (e + 305.0) / 4320.0, 0.0, -(e + 2315.0) / 1440.0, (z + 415.0) / 270.0, 0.0, 0.0},
      {-(f + 445.0) / 1440.0, (w + 7295.0) / 2160.0, -(u + 12785.0) / 4320.0, (b + 335.0) / 540.0,
       -(y + 725.0) / 540.0, (e + 2315.0) / 1440.0, 0.0, -(e + 785.0) / 4320.0, -1.0 / 12.0, 0.0},
      {-(h + 421.0) / 1296.0, -(a + 655.0) / 4320.0, (b + 335.0) / 540.0, -(a - 12085.0) / 12960.0,
       (e + 3335.0) / 4320.0, -(z + 415.0) / 270.0, (e + 785.0) / 4320.0, 0.0, 8.0 / 12.0, -1.0 / 12.0}};
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (std::fabs(M[r][col]) > std::fabs(M[piv][col])) piv = r;
    for (int m = 0; m < 10; ++m) std::swap(M[col][m], M[piv][m]);
    const double inv = 1.0 / M[col][col];
    for (int m = 0; m < 10; ++m) M[col][m] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const double t = M[r][col];
      for (int m = 0; m < 10; ++m) M[r][m] -= t * M[col][m];
    }
  }
  double wd[24];
  float wf[24];
  for (int r = 0; r < 4; ++r)
    for (int m = 0; m < 6; ++m) {
      wd[6 * r + m] = M[r][4 + m];
      wf[6 * r + m] = (float)M[r][4 + m];
    }
  cudaError_t err = cudaMemcpyToSymbol(c_carp_d, wd, sizeof(wd));
  if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_carp_f, wf, sizeof(wf));
  return err;
}

void launch2_metrics(const Ctx &c, const double *x1, cudaStream_t s, int64_t *launches) {
  dim3 b(32, 8), gr((c.g.n0 + 31) / 32, (c.g.n1 + 7) / 8);
  const double inv_d1 = 1.0 / c.plan.delta[1];
  const int cly = closure_bits(c.plan, 1);
  k2_metric_d11<<<gr, b, 0, s>>>(c.g, x1, c.d11, inv_d1, cly);
  k2_metric_halo<<<(c.g.n1 + 2 * c.hy2 + 127) / 128, 128, 0, s>>>(c.g, c.d11, 0, c.hx2, c.hy2);
  k2_metric_halo<<<(c.g.n0 + 2 * c.hx2 + 127) / 128, 128, 0, s>>>(c.g, c.d11, 1, c.hx2, c.hy2);
  k2_metric_sd<<<gr, b, 0, s>>>(c.g, c.d11, c.sd111, inv_d1, cly);
  *launches += 4;
}

void launch2_save(const Ctx &c, cudaStream_t s, int64_t *launches) {
  int nb = (int)(((int64_t)c.g.n0 * c.g.n1 + 255) / 256);
  if (nb > c.num_sms * 4) nb = c.num_sms * 4;
  k2_save<<<nb, 256, 0, s>>>(c.g, q4(c.q64_2d), q4(c.du2), 4);
  ++*launches;
}

void launch2_bcs(const Ctx &c, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  if (p.bc[0][0] == OSB_BC_PERIODIC && p.bc[1][0] == OSB_BC_PERIODIC) {  // doubly periodic: x0, then x1
    for (int d = 0; d < 2; ++d) {
      const int64_t N = (int64_t)4 * (d == 0 ? c.g.n1 + 2 * c.hy2 : c.g.n0 + 2 * c.hx2) * (d == 0 ? c.hx2 : c.hy2);
      int nb = (int)((N + 255) / 256);
      if (nb > c.num_sms * 4) nb = c.num_sms * 4;
      k2_wrap<<<nb, 256, 0, s>>>(c.g, q4(c.q64_2d), d, c.hx2, c.hy2);
    }
    *launches += 2;
    return;
  }
  BC2Args a;
  a.gama = p.gama;
  a.Minf = p.Minf;
  a.Twall = p.Twall;
  a.delta0 = p.delta[0];
  a.xs = p.dirichlet_x_switch;
  a.hx = c.hx2;
  a.hy = c.hy2;
  for (int v = 0; v < 4; ++v) {
    a.st.lo[v] = p.dirichlet_state[0][v];
    a.st.hi[v] = p.dirichlet_state[1][v];
    a.f0[v] = p.dirichlet_x0[0][v];
    a.f1[v] = p.dirichlet_x0[1][v];
  }
  a.dir0 = p.bc[0][0] == OSB_BC_DIRICHLET;
  a.dir1 = p.bc[0][1] == OSB_BC_DIRICHLET;
  a.sym0 = p.bc[1][0] == OSB_BC_SYMMETRY;
  a.sym1 = p.bc[1][1] == OSB_BC_SYMMETRY;
  a.adi0 = p.bc[0][0] == OSB_BC_ADIABATIC_WALL;
  a.adi1 = p.bc[0][1] == OSB_BC_ADIABATIC_WALL;
  a.adiy0 = p.bc[1][0] == OSB_BC_ADIABATIC_WALL;
  a.per0 = p.bc[0][0] == OSB_BC_PERIODIC;
  a.wall1 = p.bc[1][1] == OSB_BC_ISOTHERMAL_WALL;
  // rows 4 .. n1-6 to the other blocks: block 0 takes the rows a top symmetry face reads (n1-5 ..)
  const int rows = c.g.n1 - 9 > 0 ? c.g.n1 - 9 : 0, cols = c.g.n0 - 3 > 0 ? c.g.n0 - 3 : 0;
  const int row_blocks = (rows + BC2_THREADS - 1) / BC2_THREADS;
  const int col_blocks = (3 * cols + BC2_THREADS - 1) / BC2_THREADS;
  k2_bc<<<1 + row_blocks + col_blocks, BC2_THREADS, 0, s>>>(c.g, q4(c.q64_2d), a, row_blocks);
  *launches += 1;
  if (a.per0) {  // the x0 exchange after the walls, which act on single x0 columns
    const int64_t N = (int64_t)4 * (c.g.n1 + 2 * c.hy2) * c.hx2;
    int nb = (int)((N + 255) / 256);
    if (nb > c.num_sms * 4) nb = c.num_sms * 4;
    k2_wrap<<<nb, 256, 0, s>>>(c.g, q4(c.q64_2d), 0, c.hx2, c.hy2);
    *launches += 1;
  }
}

// Mixed: the FP32 working state from the FP64 master at every padded point (the right-hand side's
// k2_prims does this for its own stage; this one leaves the bound arrays current after a step).
void launch2_to_state(const Ctx &c, cudaStream_t s, int64_t *launches) {
  if (!c.mixed) return;
  int nb = (int)((c.g.numel + 255) / 256);
  if (nb > 152 * 8) nb = 152 * 8;
  k2_to_state<<<nb, 256, 0, s>>>(c.g.numel, q4(c.q64_2d), q4t<float>(c.qa));
  ++*launches;
}

template <typename T, int D>
static void launch2_flux(const Ctx &c, dim3 grid, Q4T<const T> q, Prims<const T> prc, Q4T<T> r, double eps,
                         const T *ctp, cudaStream_t s) {
  const osb_plan_desc &p = c.plan;
  const double idd = 1.0 / p.delta[D];
  // the FP64-next-to-shocks instantiation when the plan asks for it (FP32 state only)
  const bool sh = sizeof(T) == 4 && p.shock_fp64 > 0.0;
  auto launch = [&](auto plain, auto shock) {
    (sh ? shock : plain)<<<grid, 256, 0, s>>>(c.g, q, prc, c.d11, r, p.gama, eps, p.teno_ct, idd, ctp, p.shock_fp64,
                                              p.averaging == OSB_AVG_SIMPLE);
  };
  if (p.conv == OSB_CONV_TENO5)
    launch(k2_flux<T, D, SCH_TENO, false>, k2_flux<T, D, SCH_TENO, sizeof(T) == 4>);
  else if (p.conv == OSB_CONV_TENO6)
    launch(k2_flux<T, D, SCH_TENO6, false>, k2_flux<T, D, SCH_TENO6, sizeof(T) == 4>);
  else if (p.conv == OSB_CONV_WENO5Z)
    launch(k2_flux<T, D, SCH_Z, false>, k2_flux<T, D, SCH_Z, sizeof(T) == 4>);
  else
    launch(k2_flux<T, D, SCH_JS, false>, k2_flux<T, D, SCH_JS, sizeof(T) == 4>);
}

template <typename T> void launch2_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s,
                                       int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  Prims<T> pr;
  pr.u0 = static_cast<T *>(c.prim2[0]);
  pr.u1 = static_cast<T *>(c.prim2[1]);
  pr.p = static_cast<T *>(c.prim2[2]);
  pr.a = static_cast<T *>(c.prim2[3]);
  pr.T_ = static_cast<T *>(c.prim2[4]);
  pr.mu = static_cast<T *>(c.prim2[5]);
  Prims<const T> prc{pr.u0, pr.u1, pr.p, pr.a, pr.T_, pr.mu};
  Q4T<const T> q = q4t<const T>(c.qa);
  dim3 b(32, 8), gp((c.g.n0 + 8 + 31) / 32, (c.g.n1 + 8 + 7) / 8);
  k2_prims<T><<<gp, b, 0, s>>>(c.g, q4(c.q64_2d), q4t<float>(c.qa), pr, p.gama, p.Minf,
                                p.visc == OSB_VISC_CONST ? -1.0 : p.SuthT / p.RefT);
  Q4T<T> r = q4t<T>(c.res);
  const bool teno = p.conv == OSB_CONV_TENO5 || p.conv == OSB_CONV_TENO6;
  const double eps = teno ? p.teno_eps : p.weno_eps;
  const T *ctp = nullptr;
  if (teno && p.teno_adaptive) {
    Sensor2Args sa{1.0 / p.delta[0], 1.0 / p.delta[1], p.teno_a1, p.teno_a2, p.sensor_eps, closure_bits(p, 0),
                   closure_bits(p, 1)};
    dim3 gs((c.g.n0 + 2 + 31) / 32, (c.g.n1 + 2 + 7) / 8);
    k2_sensor_ct<T><<<gs, b, 0, s>>>(c.g, prc, c.d11, static_cast<T *>(c.ct2), sa);
    ctp = static_cast<const T *>(c.ct2);
    ++*launches;
  }
  // the x fluxes (this stream), the x1 fluxes and the viscous terms (side streams) read only the
  // primitives and the state and write separate arrays, so they run concurrently: each alone leaves
  // most of the GPU idle on a block of this size
  cudaEventRecord(c.ev_fork2, s);
  cudaStreamWaitEvent(c.side2[0], c.ev_fork2, 0);
  cudaStreamWaitEvent(c.side2[1], c.ev_fork2, 0);
  const bool skew = p.conv == OSB_CONV_CENTRAL_SKEW;
  if (skew) {  // central skew-symmetric convective terms (laminar_channel.py), Cartesian
    const Skew2Args sa{1.0 / p.delta[0], 1.0 / p.delta[1], closure_bits(p, 0), closure_bits(p, 1)};
    k2_skew<T><<<dim3((c.g.n0 + 31) / 32, (c.g.n1 + 7) / 8), dim3(32, 8), 0, s>>>(c.g, q, pr.u0, pr.u1, pr.p, r, sa);
  } else {
    {
      using Tl = T2Tile<0>;
      dim3 gx((c.g.n0 + Tl::TI - 2) / (Tl::TI - 1), (c.g.n1 + Tl::TA - 1) / Tl::TA);
      launch2_flux<T, 0>(c, gx, q, prc, r, eps, ctp, s);
    }
    {
      using Tl = T2Tile<1>;
      dim3 gy((c.g.n0 + Tl::TA - 1) / Tl::TA, (c.g.n1 + Tl::TI - 2) / (Tl::TI - 1));
      launch2_flux<T, 1>(c, gy, q, prc, q4t<T>(c.resy), eps, ctp, c.side2[0]);
    }
  }
  Visc2Args va;
  va.Re = p.Re;
  va.kappa = 1.0 / ((p.gama - 1) * p.Minf * p.Minf * p.Pr * p.Re);
  va.inv_d0 = 1.0 / p.delta[0];
  va.inv_d1 = 1.0 / p.delta[1];
  va.clx = closure_bits(p, 0);
  va.cly = closure_bits(p, 1);
  const bool visc = p.visc != OSB_VISC_NONE;
  Q3T<T> rv{{nullptr, nullptr, nullptr}};
  if (visc) {
    rv = Q3T<T>{{static_cast<T *>(c.resv[0]), static_cast<T *>(c.resv[1]), static_cast<T *>(c.resv[2])}};
    dim3 gv((c.g.n0 + V2X - 1) / V2X, (c.g.n1 + V2Y - 1) / V2Y);
    k2_visc<T><<<gv, dim3(V2X, V2Y), 0, c.side2[1]>>>(c.g, prc, c.d11, c.sd111, rv, va, c.hx2, c.hy2);
  }
  cudaEventRecord(c.ev_join2[0], c.side2[0]);
  cudaEventRecord(c.ev_join2[1], c.side2[1]);
  cudaStreamWaitEvent(s, c.ev_join2[0], 0);
  cudaStreamWaitEvent(s, c.ev_join2[1], 0);
  Q3T<const T> rvc{{rv.v[0], rv.v[1], rv.v[2]}};
  int nb = (int)(((int64_t)c.g.n0 * c.g.n1 + 255) / 256);
  if (nb > c.num_sms * 4) nb = c.num_sms * 4;
  Q4T<const T> ryc = q4t<const T>(c.resy);
  if (skew) ryc.v[0] = nullptr;  // the skew kernel writes the whole convective residual into res
  k2_rk<T><<<nb, 256, 0, s>>>(c.g, q4t<const T>(c.res), ryc, rvc, q4(c.du2), q4(c.q64_2d), dt, A, B, update,
                              p.rk == OSB_RK3_2REG, p.forcing[0], p.forcing[1]);
  *launches += 2 + (skew ? 1 : 2) + (visc ? 1 : 0);
}

// The adaptive TENO cut-off of the current working state over the interior, as FP64 [n1][n0]
// (the reference stores this field as TENO_B0 for output).
template <typename T> __global__ void k2_pack_ct(Grid g, const T *ct, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n0 || j >= g.n1) return;
  out[(int64_t)j * g.n0 + i] = (double)ct[g2(g, i, j)];
}

template <typename T> void launch2_cutoff(const Ctx &c, double *out, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  Prims<T> pr;
  pr.u0 = static_cast<T *>(c.prim2[0]);
  pr.u1 = static_cast<T *>(c.prim2[1]);
  pr.p = static_cast<T *>(c.prim2[2]);
  pr.a = static_cast<T *>(c.prim2[3]);
  pr.T_ = static_cast<T *>(c.prim2[4]);
  pr.mu = static_cast<T *>(c.prim2[5]);
  Prims<const T> prc{pr.u0, pr.u1, pr.p, pr.a, pr.T_, pr.mu};
  dim3 b(32, 8), gp((c.g.n0 + 8 + 31) / 32, (c.g.n1 + 8 + 7) / 8);
  k2_prims<T><<<gp, b, 0, s>>>(c.g, q4(c.q64_2d), q4t<float>(c.qa), pr, p.gama, p.Minf, p.SuthT / p.RefT);
  Sensor2Args sa{1.0 / p.delta[0], 1.0 / p.delta[1], p.teno_a1, p.teno_a2, p.sensor_eps, closure_bits(p, 0),
                   closure_bits(p, 1)};
  dim3 gs((c.g.n0 + 2 + 31) / 32, (c.g.n1 + 2 + 7) / 8);
  k2_sensor_ct<T><<<gs, b, 0, s>>>(c.g, prc, c.d11, static_cast<T *>(c.ct2), sa);
  dim3 gi((c.g.n0 + 31) / 32, (c.g.n1 + 7) / 8);
  k2_pack_ct<T><<<gi, b, 0, s>>>(c.g, static_cast<const T *>(c.ct2), out);
  *launches += 3;
}

// =============================================================================================
// span-periodic 3D wall-bounded blocks: the configuration above with a periodic x2 axis
// (apps/transitional_SBLI/transitional_SBLI.py without its body force, statistics and restart).
// The FP64 master state is the context's RK register array (qold), the working state the bound
// arrays (FP32 or FP64); the characteristic fluxes are the 3D flux kernels of osb_weno.cu, whose x1
// sweep scales its flux difference by D11(j) (Phys::ysc_d / ysc_f).  Layout: the 3D one (halos 4,
// 3, 3); the face conditions write the halo points the stencils read (the generated code also
// writes row n1+3, which no stencil reads).
// =============================================================================================
struct Q5 {
  double *v[5];
};
template <typename T> struct Q5T {
  T *v[5];
};

// Metric terms of a block stretched in x1 (one block): D11(j) = 1/(dx1/dxi1) and SD111(j) =
// dD11/dxi1 with the x1 closures (both read interior points only), and the x1 flux-difference scale
// inv_delta1 D11(j) in FP64 and as an FP32 pair.
__global__ void __launch_bounds__(256) k3w_metrics(int n1, const double *x1, double *D11, double *SD111, double *ysc_d,
                                                   float2 *ysc_f, double inv_d1, int cly) {
  for (int j = threadIdx.x; j < n1; j += blockDim.x) {
    auto G = [&](int o) { return x1[j + o]; };
    D11[j] = 1.0 / (inv_d1 * d1c<double>(G, j, n1, cly));
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n1; j += blockDim.x) {
    auto G = [&](int o) { return D11[j + o]; };
    SD111[j] = inv_d1 * d1c<double>(G, j, n1, cly);
    const double sc = inv_d1 * D11[j];
    const float hi = (float)sc;
    ysc_d[j] = sc;
    ysc_f[j] = make_float2(hi, (float)(sc - (double)hi));
  }
}

// The four faces of every interior x2 plane, one launch (blockIdx.y = plane), with the work split
// of k2_bc: block 0 of a plane applies the x faces of the rows -3..3 and n1-1..n1+2, then the y faces
// of the columns -3..0 and n0-2..n0+3; the other blocks the rows and columns between.
struct BC3Args {
  double gama, Minf, Twall, delta0, xs;
  double lo[5], hi[5];
  int ke;     // Dirichlet face keeps rhou2 and sets rhoE = state + rhou2^2/(2 rho)
  int per0;   // channel: periodic x0 (no inlet and outlet faces)
  int wall1;  // channel: isothermal wall on x1 side 1 (no Dirichlet face)
};

__device__ __forceinline__ void bc3_row(const Grid &g, const Q5 &q, const BC3Args &a, int j, int k) {
  if (a.per0) return;
  {  // inlet (inlet_pressure_extrapolate.py:11-66)
    const int64_t b = gidx(g, 0, j, k), m1 = gidx(g, -1, j, k);
    const double rhob = q.v[0][b];
    const double ub0 = fabs(q.v[1][b] / rhob), ub1 = fabs(q.v[2][b] / rhob), ub2 = fabs(q.v[3][b] / rhob);
    const double pb = (a.gama - 1) * (-0.5 * rhob * (ub0 * ub0 + ub1 * ub1 + ub2 * ub2) + q.v[4][b]);
    const double ab = sqrt(a.gama * pb / rhob);
    if (ub0 >= ab) {
      for (int v = 0; v < 5; ++v) q.v[v][b] = q.v[v][m1];
    } else {
      const double e = q.v[4][b];
      for (int t = 1; t <= 3; ++t) q.v[4][gidx(g, -t, j, k)] = e;
    }
  }
  for (int v = 0; v < 5; ++v) {  // outlet (extrapolation.py:8-58)
    const double val = q.v[v][gidx(g, g.n0 - 2, j, k)];
    for (int t = 0; t <= 4; ++t) q.v[v][gidx(g, g.n0 - 1 + t, j, k)] = val;
  }
}

// One halo point of an isothermal wall (isothermal_wall.py:32-88) whose wall row is jw and whose
// interior lies on the side sg (+1: side 0, -1: side 1) of it: the halo point jw - sg t mirrors the
// point jw + sg t with T_t = (t+1) Twall - t T(jw + sg); t = 1 also sets the wall point.
__device__ __forceinline__ void wall3_point(const Grid &g, const Q5 &q, const BC3Args &a, int i, int jw, int sg, int t,
                                            int k) {
  const double M2 = a.Minf * a.Minf, gama = a.gama;
  const int64_t w = gidx(g, i, jw, k), a1 = gidx(g, i, jw + sg, k);
  // the wall point after this face: zero momentum, energy from Twall; its pressure
  // (gama-1) (rhoE - |rhou|^2 / (2 rho)) is exactly (gama-1) rhoE there
  const double rw = q.v[0][w], ew = a.Twall * (1.0 / M2) * rw / (gama * (gama - 1.0));
  const double Pw = (gama - 1) * ew;
  const double Ta = M2 * gama * (gama - 1) *
                    (-(0.5 * q.v[1][a1] * q.v[1][a1] + 0.5 * q.v[2][a1] * q.v[2][a1] + 0.5 * q.v[3][a1] * q.v[3][a1]) /
                         q.v[0][a1] + q.v[4][a1]) /
                    q.v[0][a1];
  const int64_t m = gidx(g, i, jw + sg * t, k), hh = gidx(g, i, jw - sg * t, k);
  const double um0 = q.v[1][m] / q.v[0][m], um1 = q.v[2][m] / q.v[0][m], um2 = q.v[3][m] / q.v[0][m];
  const double Tt = (t + 1) * a.Twall - t * Ta;
  const double rh = M2 * gama * Pw / Tt;
  q.v[0][hh] = rh;
  q.v[1][hh] = -rh * um0;
  q.v[2][hh] = -rh * um1;
  q.v[3][hh] = -rh * um2;
  q.v[4][hh] = (1.0 / (gama - 1)) * Pw + 0.5 * rh * (um0 * um0 + um1 * um1 + um2 * um2);
  if (t == 1) {
    q.v[1][w] = 0.0;
    q.v[2][w] = 0.0;
    q.v[3][w] = 0.0;
    q.v[4][w] = ew;
  }
}

__device__ __forceinline__ void bc3_col(const Grid &g, const Q5 &q, const BC3Args &a, int i, int t, int k) {
  wall3_point(g, q, a, i, 0, 1, t, k);
  if (a.wall1) {  // the channel's second wall (rows n1-1 .. n1+2; the generated code's row n1+3 is never read)
    wall3_point(g, q, a, i, g.n1 - 1, -1, t, k);
  } else if (t == 1) {
    const double x0 = a.delta0 * i;  // Dirichlet top face
    const double *st = x0 > a.xs ? a.hi : a.lo;
    for (int j = g.n1 - 1; j < g.n1 + HY; ++j) {
      const int64_t m = gidx(g, i, j, k);
      if (a.ke) {  // rho, rhou0, rhou1 set; rhoE from the face's rho and the local rhou2
        for (int v = 0; v < 3; ++v) q.v[v][m] = st[v];
        q.v[4][m] = st[4] + 0.5 * (q.v[3][m] * q.v[3][m]) / q.v[0][m];
      } else {
        for (int v = 0; v < 5; ++v) q.v[v][m] = st[v];
      }
    }
  }
}

__global__ void __launch_bounds__(BC2_THREADS) k3w_bc(Grid g, Q5 q, BC3Args a, int row_blocks) {
  const int tid = threadIdx.x, k = blockIdx.y;
  if (blockIdx.x == 0) {
    for (int j = -3 + tid; j < g.n1 + HY; j += BC2_THREADS)
      if (j <= 3 || j >= g.n1 - 1) bc3_row(g, q, a, j, k);
    __syncthreads();
    for (int w = tid; w < 3 * (g.n0 + HX + 3); w += BC2_THREADS) {
      const int i = w / 3 - 3;
      if (i <= 0 || i >= g.n0 - 2) bc3_col(g, q, a, i, w % 3 + 1, k);
    }
  } else if ((int)blockIdx.x <= row_blocks) {
    const int j = 4 + ((int)blockIdx.x - 1) * BC2_THREADS + tid;
    if (j < g.n1 - 1) bc3_row(g, q, a, j, k);
  } else {
    const int w = ((int)blockIdx.x - 1 - row_blocks) * BC2_THREADS + tid;
    const int i = 1 + w / 3;
    if (i < g.n0 - 2) bc3_col(g, q, a, i, w % 3 + 1, k);
  }
}

// Periodic x0 of a channel block (exchange.py:9-57) on the interior planes, after the wall faces
// (which act on single x0 columns, so the order does not change a value): columns -4..-1 take
// n0-4..n0-1 and columns n0..n0+3 take 0..3, every padded row.
__global__ void k3w_wrapx(Grid g, Q5 q) {
  const int rows = g.n1 + 2 * HY;
  const int64_t N = (int64_t)rows * g.n2 * HX;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 5 * N; t += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / N);
    const int64_t e = t % N;
    const int x = (int)(e % HX), j = (int)((e / HX) % rows) - HY, k = (int)(e / ((int64_t)HX * rows));
    double *f = q.v[v];
    f[gidx(g, x - HX, j, k)] = f[gidx(g, g.n0 - HX + x, j, k)];
    f[gidx(g, g.n0 + x, j, k)] = f[gidx(g, x, j, k)];
  }
}

// Periodic x2 (exchange.py:9-57): planes -3..-1 take n2-3..n2-1 and planes n2..n2+2 take 0..2,
// whole padded x0-x1 planes.
__global__ void k3w_wrap(Grid g, Q5 q) {
  const int64_t plane = g.sz, N = plane * HZ;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 5 * N; t += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(t / N);
    const int64_t e = t % N, zo = e / plane, o = e % plane;  // zo = 0..HZ-1
    double *f = q.v[v];
    f[o + zo * plane] = f[o + (g.n2 + zo) * plane];                        // plane zo - HZ <- n2 + zo - HZ
    f[o + (HZ + g.n2 + zo) * plane] = f[o + (HZ + zo) * plane];           // plane n2 + zo <- zo
  }
}

// FP64 master -> working state over every padded point
template <typename T> __global__ void k3w_to_state(int64_t numel, Q5 src, Q5T<T> dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < numel; t += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if constexpr (sizeof(T) == 4) dst.v[v][t] = cvt_f64_f32(src.v[v][t]);
      else dst.v[v][t] = src.v[v][t];
    }
}

// Viscous terms (momentum 0..2, energy) at every interior point, as k2_visc with the third
// component and the periodic x2 derivatives (and x0 ones on channel blocks), mu from Sutherland's law
// or, with vexp > 0, the power law T^vexp (turbulent_channel.py:30): d/dx1 = D11 d/dxi1, d2/dx1^2 = D11^2 d2/dxi1^2 +
// D11 SD111 d/dxi1, mixed derivatives nest first derivatives (the inner x0 or x2 derivative over the
// extended range of the outer axis).  A block marches a 32 x 8 x-x1 tile through kz planes in x2: a
// ring of five planes in dynamic shared memory holds u0, u1, u2, T and mu of the planes k-2..k+2 with
// V2H points around the tile in x0 and x1, one plane staged per step; the primitives are formed from
// the working state as they are staged (FP32: u, p and T rounded once, prims_f32).
constexpr int VISC3_KZ = 8;  // x2 planes per block of the viscous kernel
template <typename T> constexpr size_t visc3_smem() {
  return sizeof(T) * 5 * 5 * (size_t)(V2Y + 2 * V2H) * (V2X + 2 * V2H);
}

template <typename T>
__global__ void __launch_bounds__(V2X * V2Y, sizeof(T) == 4 ? 3 : 1) k3w_visc(Grid g, Q5T<const T> q, const double *D11, const double *SD111,
                                                      Q5T<T> rv, Visc2Args va, double gama, double gM2, double suth,
                                                      double vexp, int clx, int cly, int kz) {
  constexpr int SX = V2X + 2 * V2H, SY = V2Y + 2 * V2H, PL = SX * SY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sm = reinterpret_cast<T *>(smem_raw);  // [field u0 u1 u2 T mu][ring slot: plane mod 5][SY][SX]
  auto R = [&](int f, int slot, int y, int x) -> T & { return sm[((f * 5 + slot) * SY + y) * SX + x]; };
  const int i0 = blockIdx.x * V2X, j0 = blockIdx.y * V2Y, k0 = (int)blockIdx.z * kz;
  const int k1 = k0 + kz < g.n2 ? k0 + kz : g.n2;
  const int tid = threadIdx.y * V2X + threadIdx.x;
  const T S1 = T(suth);
  auto stage = [&](int gk) {  // plane gk (>= -2) into ring slot (gk + 5) mod 5
    const int slot = (gk + 5) % 5;
    for (int t = tid; t < PL; t += V2X * V2Y) {
      const int r = t, li = r % SX, lj = r / SX;
      const int gi = i0 - V2H + li, gj = j0 - V2H + lj;
      if (gi < -HX || gi >= g.n0 + HX || gj < -HY || gj >= g.n1 + HY) continue;
      const int64_t m = gidx(g, gi, gj, gk);
      T u[3], p, Tt;
      const T rho = q.v[0][m];
      if constexpr (sizeof(T) == 4) {
        const float gm1 = (float)(gama - 1.0), gm1_lo = (float)((gama - 1.0) - (double)gm1);
        float ir, p_lo;
        prims_f32(rho, q.v[1][m], q.v[2][m], q.v[3][m], q.v[4][m], gm1, gm1_lo, ir, u, p, p_lo);
        Tt = scaled_ratio_f32((float)gM2, p, p_lo, rho, ir);
      } else {
        const T ir = T(1) / rho;
#pragma unroll
        for (int c = 0; c < 3; ++c) u[c] = q.v[1 + c][m] * ir;
        p = (T(gama) - T(1)) * (q.v[4][m] - T(0.5) * rho * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
        Tt = T(gM2) * p * ir;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) R(c, slot, lj, li) = u[c];
      R(3, slot, lj, li) = Tt;
      R(4, slot, lj, li) = vexp > 0.0 ? pow_t(Tt, T(vexp)) : (S1 + T(1)) * Tt * sqrt_t(Tt) / (S1 + Tt);
    }
  };
  for (int gk = k0 - 2; gk < k0 + 2; ++gk) stage(gk);
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const int li = threadIdx.x + V2H, lj = threadIdx.y + V2H;
  for (int k = k0; k < k1; ++k) {
    stage(k + 2);
    __syncthreads();
    int sl[5];
#pragma unroll
    for (int z = 0; z < 5; ++z) sl[z] = (k + z + 3) % 5;  // slot of plane k - 2 + z
    auto S = [&](int f, int z, int y, int x) -> T & { return R(f, sl[z], y, x); };
    if (i < g.n0 && j < g.n1) {
      const int64_t c = gidx(g, i, j, k);
      const T id0 = T(va.inv_d0), id1 = T(va.inv_d1), id2 = T(va.inv_d2), iRe = T(1.0 / va.Re);
      const T Dm = T(D11[j]), Sm = T(SD111[j]), mu = S(4, 2, lj, li);
      const T c1 = T(1.0 / 12.0), c2 = T(2.0 / 3.0);
      // central first derivative along x2 of the value at plane offset z (periodic: no closure)
      auto dz1 = [&](auto &&F) { return id2 * (c1 * F(-2) - c2 * F(-1) + c2 * F(1) - c1 * F(2)); };
      auto dz2 = [&](auto &&F) {
        return id2 * id2 * (-c1 * F(-2) + T(4.0 / 3.0) * F(-1) - T(2.5) * F(0) + T(4.0 / 3.0) * F(1) - c1 * F(2));
      };
      T gr[3][3], h[3][3][3];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        auto X = [&](int o) { return S(f, 2, lj, li + o); };
        auto Y = [&](int o) { return S(f, 2, lj + o, li); };
        auto Z = [&](int o) { return S(f, 2 + o, lj, li); };
        gr[f][0] = id0 * d1c<T>(X, i, g.n0, clx);
        const T fy = id1 * d1c<T>(Y, j, g.n1, cly);
        gr[f][1] = Dm * fy;
        gr[f][2] = dz1(Z);
        h[f][0][0] = id0 * id0 * d2c<T>(X, i, g.n0, clx);
        h[f][1][1] = Dm * Dm * (id1 * id1 * d2c<T>(Y, j, g.n1)) + Dm * Sm * fy;
        h[f][2][2] = dz2(Z);
        // x0 derivative of row j+o / of plane k+o, then the outer derivative
        auto inner_xy = [&](int o) { return id0 * d1c<T>([&](int p) { return S(f, 2, lj + o, li + p); }, i, g.n0, clx); };
        auto inner_xz = [&](int o) { return id0 * d1c<T>([&](int p) { return S(f, 2 + o, lj, li + p); }, i, g.n0, clx); };
        auto inner_zy = [&](int o) { return dz1([&](int p) { return S(f, 2 + p, lj + o, li); }); };
        h[f][0][1] = h[f][1][0] = Dm * (id1 * d1c<T>(inner_xy, j, g.n1, cly));
        h[f][0][2] = h[f][2][0] = dz1(inner_xz);
        h[f][1][2] = h[f][2][1] = Dm * (id1 * d1c<T>(inner_zy, j, g.n1, cly));
      }
      auto XT = [&](int o) { return S(3, 2, lj, li + o); };
      auto YT = [&](int o) { return S(3, 2, lj + o, li); };
      auto ZT = [&](int o) { return S(3, 2 + o, lj, li); };
      auto Xmu = [&](int o) { return S(4, 2, lj, li + o); };
      auto Ymu = [&](int o) { return S(4, 2, lj + o, li); };
      auto Zmu = [&](int o) { return S(4, 2 + o, lj, li); };
      const T mug[3] = {id0 * d1c<T>(Xmu, i, g.n0, clx), Dm * id1 * d1c<T>(Ymu, j, g.n1, cly), dz1(Zmu)};
      const T Tyx = id1 * d1c<T>(YT, j, g.n1, cly);
      const T Tg[3] = {id0 * d1c<T>(XT, i, g.n0, clx), Dm * Tyx, dz1(ZT)};
      const T Tlap = id0 * id0 * d2c<T>(XT, i, g.n0, clx) + (Dm * Dm * (id1 * id1 * d2c<T>(YT, j, g.n1)) + Dm * Sm * Tyx) + dz2(ZT);
      const T div = gr[0][0] + gr[1][1] + gr[2][2];
      const T uu[3] = {S(0, 2, lj, li), S(1, 2, lj, li), S(2, 2, lj, li)};
      T e = T(va.kappa) * (mu * Tlap + mug[0] * Tg[0] + mug[1] * Tg[1] + mug[2] * Tg[2]);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        T v = T(0);
#pragma unroll
        for (int b = 0; b < 3; ++b) v += mug[b] * (gr[a][b] + gr[b][a] - (a == b ? T(2.0 / 3.0) * div : T(0))) * iRe;
        const T lap = h[a][0][0] + h[a][1][1] + h[a][2][2];
        const T ddiv = h[0][a][0] + h[1][a][1] + h[2][a][2];
        v += mu * iRe * (lap + ddiv * T(1.0 / 3.0));
        rv.v[a][c] = v;
        e += uu[a] * v;
#pragma unroll
        for (int b = 0; b < 3; ++b) e += mu * iRe * (gr[a][b] + gr[b][a] - (a == b ? T(2.0 / 3.0) * div : T(0))) * gr[a][b];
      }
      rv.v[3][c] = e;
    }
    __syncthreads();  // before the next plane overwrites the slot of plane k - 2
  }
}

// R = fluxes + viscous terms at every interior point, then the LS-RK3 update of the FP64 master
// (update = 1), or R itself into du (update = 0)
// body force of the continuity equation: bf_xy[j][i] = A exp(-((x0-xF)^2 + (x1-yF)^2)), bf_z[k] =
// cos(bta x2), *bf_t = sin(omega dt iter) of the current step (null bf_xy: none)
struct BF3 {
  const double *xy, *z, *t;
};
// the channel's constant forcing c_j (turbulent_channel.py:15-16): -c_i in the momentum equations,
// -c_j u_j in the energy equation, u_j from the FP64 state the stage started from (on = 0: none)
struct Force3 {
  double c[3];
  int on;
};

template <typename T>
__global__ void k3w_rk(Grid g, Q5T<const T> rf, Q5T<const T> rv, Q5 du, Q5 q64, double dt, double A, double B,
                       int update, BF3 bf, Force3 fo) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    const int64_t c = gidx(g, i, j, k);
    T R[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) R[v] = rf.v[v][c];
#pragma unroll
    for (int v = 1; v < 5; ++v) R[v] += rv.v[v - 1][c];
    if (bf.xy) R[0] += T(bf.xy[(int64_t)j * g.n0 + i] * bf.z[k] * bf.t[0]);
    double Rd[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) Rd[v] = to_f64(R[v]);
    if (fo.on) {
      const double ir = 1.0 / q64.v[0][c];
      Rd[4] -= fo.c[0] * (q64.v[1][c] * ir) + fo.c[1] * (q64.v[2][c] * ir) + fo.c[2] * (q64.v[3][c] * ir);
#pragma unroll
      for (int d = 0; d < 3; ++d) Rd[1 + d] -= fo.c[d];
    }
    if (update) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double d = dt * Rd[v] + A * du.v[v][c];
        du.v[v][c] = d;
        q64.v[v][c] = B * d + q64.v[v][c];
      }
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) du.v[v][c] = Rd[v];
    }
  }
}

// Modified Ducros sensor of a wall-bounded block (shock_sensors.py:12-49 with the metric, as
// generated for transitional_SBLI.py) and the adaptive TENO cut-off (teno.py:430-443) over the
// points [-1, n_d] of every axis: on the interior, u_i = rhou_i/rho with the x0 and x1 closures and
// d/dx1 = D11 d/dxi1, theta = (1/2 - 1/2 tanh(250 div + 2.5)) div^2 / (eps + |curl u|^2 + div^2);
// theta = 0 elsewhere; C_T = 10^-floor(a1 - a2 (1 - (1 - theta)^4 (1 + 4 theta))) from the table of
// correctly rounded powers (FP64 exponent, as the 2D kernel).
template <typename T>
__global__ void k3w_sensor(Grid g, Q5T<const T> q, const double *D11, T *ct, Sensor2Args sa, double inv_d2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - 1, j = blockIdx.y * blockDim.y + threadIdx.y - 1;
  const int k = (int)blockIdx.z - 1;
  if (i > g.n0 || j > g.n1) return;
  const int64_t n = gidx(g, i, j, k);
  double th = 0.0;
  if (i >= 0 && i < g.n0 && j >= 0 && j < g.n1 && k >= 0 && k < g.n2) {
    auto U = [&](int c, int di, int dj, int dk) {
      const int64_t m = gidx(g, i + di, j + dj, k + dk);
      return q.v[1 + c][m] / q.v[0][m];
    };
    const T id0 = T(sa.inv_d0), id1 = T(sa.inv_d1), id2 = T(inv_d2), Dm = T(D11[j]);
    T du[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      du[c][0] = id0 * d1c<T>([&](int o) { return U(c, o, 0, 0); }, i, g.n0, sa.clx);
      du[c][1] = Dm * (id1 * d1c<T>([&](int o) { return U(c, 0, o, 0); }, j, g.n1, sa.cly));
      du[c][2] = id2 * (T(1.0 / 12.0) * U(c, 0, 0, -2) - T(2.0 / 3.0) * U(c, 0, 0, -1) +
                        T(2.0 / 3.0) * U(c, 0, 0, 1) - T(1.0 / 12.0) * U(c, 0, 0, 2));
    }
    const T div = du[0][0] + du[1][1] + du[2][2];
    const T w0 = du[2][1] - du[1][2], w1 = du[0][2] - du[2][0], w2 = du[1][0] - du[0][1];
    const T sw = T(0.5) - T(0.5) * tanh_t(T(250) * div + T(2.5));
    th = (double)(sw * (div * div) / (T(sa.eps) + w0 * w0 + w1 * w1 + w2 * w2 + div * div));
  }
  const double w = 1.0 - th;
  const double e = floor(sa.a1 - sa.a2 * (1.0 - (w * w) * (w * w) * (4.0 * th + 1.0)));
  ct[n] = T((e >= 0.0 && e <= 22.0) ? c_p10n[(int)e] : pow(10.0, -e));
}

// the body-force tables of a block (once, after the coordinates): bf_xy and bf_z
__global__ void k3w_bf_tables(Grid g, const double *x1, double delta0, double delta2, double A, double xF, double yF,
                              double bta, double *xy, double *z) {
  const int64_t N = (int64_t)g.n0 * g.n1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N + g.n2; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < N) {
      const int i = (int)(t % g.n0), j = (int)(t / g.n0);
      const double x0 = delta0 * i, y = x1[j];
      xy[t] = A * exp(-(x0 - xF) * (x0 - xF) - (y - yF) * (y - yF));
    } else {
      const int k = (int)(t - N);
      z[k] = cos(bta * (delta2 * k));
    }
  }
}

// the body force's time factor sin(omega dt iter) at the start of a step (advance = 0), the step
// count at its end (advance = 1)
__global__ void k3w_tick(long long *iter, double *t, double omega_dt, int advance) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (advance) ++iter[0];
    else t[0] = sin(omega_dt * (double)iter[0]);
  }
}

static Q5 q5(double *const *a) {
  Q5 r;
  for (int v = 0; v < 5; ++v) r.v[v] = a[v];
  return r;
}
template <typename T> static Q5T<T> q5t(void *const *a) {
  Q5T<T> r;
  for (int v = 0; v < 5; ++v) r.v[v] = static_cast<T *>(a[v]);
  return r;
}

void launch3w_metrics(const Ctx &c, const double *x1_line, cudaStream_t s, int64_t *launches) {
  k3w_metrics<<<1, 256, 0, s>>>(c.g.n1, x1_line, c.d11, c.sd111, c.ysc_d, c.ysc_f, 1.0 / c.plan.delta[1],
                                closure_bits(c.plan, 1));
  ++*launches;
}

// face conditions (and the x0 wrap of a channel block) and the x2 wrap on the FP64 master, then the
// working state from it
template <typename T> void launch3w_bcs(const Ctx &c, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  BC3Args a;
  a.gama = p.gama;
  a.Minf = p.Minf;
  a.Twall = p.Twall;
  a.delta0 = p.delta[0];
  a.xs = p.dirichlet_x_switch;
  for (int v = 0; v < 5; ++v) {
    a.lo[v] = p.dirichlet_state[0][v];
    a.hi[v] = p.dirichlet_state[1][v];
  }
  a.ke = p.dirichlet_ke;
  a.per0 = p.bc[0][0] == OSB_BC_PERIODIC;
  a.wall1 = p.bc[1][1] == OSB_BC_ISOTHERMAL_WALL;
  const int rows = (c.g.n1 - 5 > 0 && !a.per0) ? c.g.n1 - 5 : 0, cols = c.g.n0 - 3 > 0 ? c.g.n0 - 3 : 0;
  const int row_blocks = (rows + BC2_THREADS - 1) / BC2_THREADS;
  const int col_blocks = (3 * cols + BC2_THREADS - 1) / BC2_THREADS;
  k3w_bc<<<dim3(1 + row_blocks + col_blocks, c.g.n2), BC2_THREADS, 0, s>>>(c.g, q5(c.qold), a, row_blocks);
  int nb;
  if (a.per0) {
    nb = (int)((5 * (int64_t)(c.g.n1 + 2 * HY) * c.g.n2 * HX + 255) / 256);
    if (nb > c.num_sms * 8) nb = c.num_sms * 8;
    k3w_wrapx<<<nb, 256, 0, s>>>(c.g, q5(c.qold));
    ++*launches;
  }
  nb = (int)((5 * c.g.sz * HZ + 255) / 256);
  if (nb > c.num_sms * 8) nb = c.num_sms * 8;
  k3w_wrap<<<nb, 256, 0, s>>>(c.g, q5(c.qold));
  nb = (int)((c.g.numel + 255) / 256);
  if (nb > c.num_sms * 8) nb = c.num_sms * 8;
  k3w_to_state<T><<<nb, 256, 0, s>>>(c.g.numel, q5(c.qold), q5t<T>(c.qa));
  *launches += 3;
}

// One stage's right-hand side: the x0, x1, x2 flux passes into res (this stream) and the viscous
// terms into resv (a side stream) concurrently, then R and the LS-RK3 update (or R into du).
template <typename T>
void launch3w_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  Fields5<const T> q;
  Fields5<T> r;
  for (int v = 0; v < 5; ++v) {
    q.v[v] = static_cast<const T *>(c.qa[v]);
    r.v[v] = static_cast<T *>(c.res[v]);
  }
  if (p.teno_adaptive) {  // the cut-off of every interface from the sensor of the working state
    Sensor2Args sa{1.0 / p.delta[0], 1.0 / p.delta[1], p.teno_a1, p.teno_a2, p.sensor_eps, closure_bits(p, 0),
                   closure_bits(p, 1)};
    dim3 b(32, 8), gs((c.g.n0 + 2 + 31) / 32, (c.g.n1 + 2 + 7) / 8, c.g.n2 + 2);
    k3w_sensor<T><<<gs, b, 0, s>>>(c.g, q5t<const T>(c.qa), c.d11, static_cast<T *>(c.ct2), sa, 1.0 / p.delta[2]);
    ++*launches;
  }
  cudaEventRecord(c.ev_fork2, s);
  cudaStreamWaitEvent(c.side2[1], c.ev_fork2, 0);
  for (int d = 0; d < 3; ++d) launch_weno_dir<T>(c, q, r, d, s, launches);
  Visc2Args va;
  va.Re = p.Re;
  va.kappa = 1.0 / ((p.gama - 1) * p.Minf * p.Minf * p.Pr * p.Re);
  va.inv_d0 = 1.0 / p.delta[0];
  va.inv_d1 = 1.0 / p.delta[1];
  va.inv_d2 = 1.0 / p.delta[2];
  Q5T<T> rv{{static_cast<T *>(c.resv[0]), static_cast<T *>(c.resv[1]), static_cast<T *>(c.resv[2]),
             static_cast<T *>(c.resv[3]), nullptr}};
  const int kz = VISC3_KZ;
  dim3 gv((c.g.n0 + V2X - 1) / V2X, (c.g.n1 + V2Y - 1) / V2Y, (c.g.n2 + kz - 1) / kz);
  k3w_visc<T><<<gv, dim3(V2X, V2Y), visc3_smem<T>(), c.side2[1]>>>(
      c.g, q5t<const T>(c.qa), c.d11, c.sd111, rv, va, p.gama, p.gama * p.Minf * p.Minf, p.SuthT / p.RefT,
      p.visc == OSB_VISC_POWER ? p.visc_exp : 0.0, closure_bits(p, 0), closure_bits(p, 1), kz);
  cudaEventRecord(c.ev_join2[1], c.side2[1]);
  cudaStreamWaitEvent(s, c.ev_join2[1], 0);
  Q5T<const T> rf{{r.v[0], r.v[1], r.v[2], r.v[3], r.v[4]}};
  Q5T<const T> rvc{{rv.v[0], rv.v[1], rv.v[2], rv.v[3], nullptr}};
  int nb = (int)(((int64_t)c.g.n0 * c.g.n1 * c.g.n2 + 255) / 256);
  if (nb > c.num_sms * 8) nb = c.num_sms * 8;
  const BF3 bf{c.bf_xy, c.bf_z, c.bf_t};
  const Force3 fo{{p.forcing[0], p.forcing[1], p.forcing[2]},
                  p.forcing[0] != 0.0 || p.forcing[1] != 0.0 || p.forcing[2] != 0.0};
  k3w_rk<T><<<nb, 256, 0, s>>>(c.g, rf, rvc, q5(c.du2), q5(c.qold), dt, A, B, update, bf, fo);
  *launches += 2;
}

void launch3w_bf_tables(const Ctx &c, cudaStream_t s, int64_t *launches) {
  if (!c.bf_xy) return;
  const osb_plan_desc &p = c.plan;
  const int64_t N = (int64_t)c.g.n0 * c.g.n1 + c.g.n2;
  int nb = (int)((N + 255) / 256);
  if (nb > c.num_sms * 8) nb = c.num_sms * 8;
  k3w_bf_tables<<<nb, 256, 0, s>>>(c.g, c.x1, p.delta[0], p.delta[2], p.body_force[0], p.body_force[1],
                                   p.body_force[2], p.body_force[3], c.bf_xy, c.bf_z);
  ++*launches;
}

// advance = 0: the time factor of the current step (start of a step); 1: count the step (its end)
void launch3w_tick(const Ctx &c, int advance, double dt, cudaStream_t s, int64_t *launches) {
  if (!c.bf_xy) return;
  k3w_tick<<<1, 32, 0, s>>>(c.d_iter, c.bf_t, c.plan.body_force[4] * dt, advance);
  ++*launches;
}

// the adaptive cut-off of the current state over the interior, FP64 [z][y][x]
template <typename T> __global__ void k3w_pack_ct(Grid g, const T *ct, double *out) {
  const int64_t N = (int64_t)g.n0 * g.n1 * g.n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.n0), j = (int)((t / g.n0) % g.n1), k = (int)(t / ((int64_t)g.n0 * g.n1));
    out[t] = (double)ct[gidx(g, i, j, k)];
  }
}

template <typename T> void launch3w_cutoff(const Ctx &c, double *out, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  launch3w_bcs<T>(c, s, launches);
  Sensor2Args sa{1.0 / p.delta[0], 1.0 / p.delta[1], p.teno_a1, p.teno_a2, p.sensor_eps, closure_bits(p, 0),
                 closure_bits(p, 1)};
  dim3 b(32, 8), gs((c.g.n0 + 2 + 31) / 32, (c.g.n1 + 2 + 7) / 8, c.g.n2 + 2);
  k3w_sensor<T><<<gs, b, 0, s>>>(c.g, q5t<const T>(c.qa), c.d11, static_cast<T *>(c.ct2), sa, 1.0 / p.delta[2]);
  int nb = (int)(((int64_t)c.g.n0 * c.g.n1 * c.g.n2 + 255) / 256);
  if (nb > c.num_sms * 8) nb = c.num_sms * 8;
  k3w_pack_ct<T><<<nb, 256, 0, s>>>(c.g, static_cast<const T *>(c.ct2), out);
  *launches += 2;
}
template void launch3w_cutoff<float>(const Ctx &, double *, cudaStream_t, int64_t *);
template void launch3w_cutoff<double>(const Ctx &, double *, cudaStream_t, int64_t *);

template <typename T> void setup3w() {
  cudaFuncSetAttribute(k3w_visc<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)visc3_smem<T>());
}

template void setup3w<float>();
template void setup3w<double>();
template void launch3w_bcs<float>(const Ctx &, cudaStream_t, int64_t *);
template void launch3w_bcs<double>(const Ctx &, cudaStream_t, int64_t *);
template void launch3w_rhs<float>(const Ctx &, int, double, double, double, cudaStream_t, int64_t *);
template void launch3w_rhs<double>(const Ctx &, int, double, double, double, cudaStream_t, int64_t *);

template void launch2_cutoff<float>(const Ctx &, double *, cudaStream_t, int64_t *);
template void launch2_cutoff<double>(const Ctx &, double *, cudaStream_t, int64_t *);

template void launch2_rhs<float>(const Ctx &, int, double, double, double, cudaStream_t, int64_t *);
template void launch2_rhs<double>(const Ctx &, int, double, double, double, cudaStream_t, int64_t *);

// =============================================================================================
// 1D Euler blocks (apps/Sod_shock_tube/Sod_shock_tube.py, apps/shu_osher/shu_osher.py): FP64, the
// three conserved arrays (rho, rhou0, rhoE) on the 2D layout with a single row.  Per stage one thread
// per interface forms the characteristic flux from the six points around it and the reference's 1D
// eigensystem (physical_models/euler_eigensystem.py:57-76: waves u-a, u, u+a, REV = [[1,1,1],
// [u-a,u,u+a],[H-ua,u^2/2,H+ua]], H = a^2/(gama-1) + u^2/2, LEV its inverse) at the Roe or simple
// average; a second launch differences the fluxes and applies the LS-RK3 update.  The blocks of these
// apps hold a few hundred to a few thousand points, so the step is launch-bound: it is one graph.
// =============================================================================================
struct Euler1Args {
  double gama, eps, ct;
  int simple;
};

template <int SCH> __global__ void __launch_bounds__(128) k1_flux(Grid g, Q4 q, Q4 flux, Euler1Args a) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 1;  // the interface i + 1/2, i = -1 .. n0-1
  if (i >= g.n0) return;
  const double gm1 = a.gama - 1.0;
  double Q[6][3], u[6], p[6], c[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int64_t m = g2(g, i + t - 2, 0);
#pragma unroll
    for (int v = 0; v < 3; ++v) Q[t][v] = q.v[v][m];
    u[t] = Q[t][1] / Q[t][0];
    p[t] = gm1 * (Q[t][2] - 0.5 * Q[t][0] * u[t] * u[t]);
    c[t] = sqrt(a.gama * p[t] / Q[t][0]);
  }
  double ua, aa;
  if (a.simple) {  // SimpleAverage (averaging.py:31-59)
    ua = 0.5 * (u[2] + u[3]);
    aa = 0.5 * (c[2] + c[3]);
  } else {  // RoeAverage (averaging.py:62-114)
    const double sl = sqrt(Q[2][0]), sr = sqrt(Q[3][0]), inv = 1.0 / (sl + sr);
    ua = inv * (sl * u[2] + sr * u[3]);
    const double Hh = inv * ((p[2] + Q[2][2]) / sl + (p[3] + Q[3][2]) / sr);
    aa = sqrt(gm1 * (Hh - 0.5 * ua * ua));
  }
  const double ia = 1.0 / aa, Hs = aa * aa / gm1 + 0.5 * ua * ua;
  const double L[3][3] = {{0.25 * ua * ia * (gm1 * ua * ia + 2.0), -0.5 * ia * (gm1 * ua * ia + 1.0), 0.5 * gm1 * ia * ia},
                          {1.0 - 0.5 * gm1 * ua * ua * ia * ia, gm1 * ua * ia * ia, -gm1 * ia * ia},
                          {0.25 * ua * ia * (gm1 * ua * ia - 2.0), -0.5 * ia * (gm1 * ua * ia - 1.0), 0.5 * gm1 * ia * ia}};
  double rec[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    double cf[6], cs[6], lam = 0.0;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const double F0 = Q[t][1], F1 = Q[t][1] * u[t] + p[t], F2 = (p[t] + Q[t][2]) * u[t];
      cf[t] = L[r][0] * F0 + L[r][1] * F1 + L[r][2] * F2;
      cs[t] = L[r][0] * Q[t][0] + L[r][1] * Q[t][1] + L[r][2] * Q[t][2];
      lam = fmax(lam, fabs(r == 0 ? c[t] - u[t] : r == 1 ? u[t] : c[t] + u[t]));
    }
    double fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    rec[r] = recon2<double, SCH>(fp, fm, a.eps, a.ct);
  }
  const int64_t n = g2(g, i, 0);
  flux.v[0][n] = rec[0] + rec[1] + rec[2];
  flux.v[1][n] = (ua - aa) * rec[0] + ua * rec[1] + (ua + aa) * rec[2];
  flux.v[2][n] = (Hs - ua * aa) * rec[0] + 0.5 * ua * ua * rec[1] + (Hs + ua * aa) * rec[2];
}

// R = -(F_i - F_{i-1}) / delta0 and the LS-RK3 update (update = 1), or R into du (update = 0)
__global__ void k1_rk(Grid g, Q4 flux, Q4 du, Q4 q, double inv_d0, double dt, double A, double B, int update) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= g.n0) return;
  const int64_t n = g2(g, i, 0);
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const double R = -(flux.v[v][n] - flux.v[v][n - 1]) * inv_d0;
    if (update) {
      const double d = dt * R + A * du.v[v][n];
      du.v[v][n] = d;
      q.v[v][n] = B * d + q.v[v][n];
    } else {
      du.v[v][n] = R;
    }
  }
}

// DirichletBC (dirichlet.py:6-41) at both ends: points -3..0 and n0-1..n0+3 take the faces' states;
// side 1 may instead extrapolate point n0-2 (extrapolation.py:8-58)
struct Faces1 {
  double f0[3], f1[3];
};
__global__ void k1_bc(Grid g, Q4 q, Faces1 f, int extrap1) {
  const int t = threadIdx.x;
  if (t < 4) {
    for (int v = 0; v < 3; ++v) q.v[v][g2(g, t - 3, 0)] = f.f0[v];
  } else if (t < 9) {
    const int i = g.n0 - 1 + (t - 4);
    for (int v = 0; v < 3; ++v) q.v[v][g2(g, i, 0)] = extrap1 ? q.v[v][g2(g, g.n0 - 2, 0)] : f.f1[v];
  }
}

void launch1_bcs(const Ctx &c, cudaStream_t s, int64_t *launches) {
  Faces1 f;
  for (int v = 0; v < 3; ++v) {
    f.f0[v] = c.plan.dirichlet_x0[0][v];
    f.f1[v] = c.plan.dirichlet_x0[1][v];
  }
  k1_bc<<<1, 32, 0, s>>>(c.g, q4(c.q64_2d), f, c.plan.bc[0][1] == OSB_BC_EXTRAPOLATION);
  ++*launches;
}

void launch1_rhs(const Ctx &c, int update, double A, double B, double dt, cudaStream_t s, int64_t *launches) {
  const osb_plan_desc &p = c.plan;
  const bool teno = p.conv == OSB_CONV_TENO5 || p.conv == OSB_CONV_TENO6;
  const Euler1Args a{p.gama, teno ? p.teno_eps : p.weno_eps, p.teno_ct, p.averaging == OSB_AVG_SIMPLE};
  const int nb = (c.g.n0 + 1 + 127) / 128;
  const Q4 q = q4(c.q64_2d);
  Q4 fl;  // the interface fluxes (the residual arrays of the context, FP64 for these blocks)
  for (int v = 0; v < 4; ++v) fl.v[v] = static_cast<double *>(c.res[v]);
  if (p.conv == OSB_CONV_TENO5) k1_flux<SCH_TENO><<<nb, 128, 0, s>>>(c.g, q, fl, a);
  else if (p.conv == OSB_CONV_TENO6) k1_flux<SCH_TENO6><<<nb, 128, 0, s>>>(c.g, q, fl, a);
  else if (p.conv == OSB_CONV_WENO5Z) k1_flux<SCH_Z><<<nb, 128, 0, s>>>(c.g, q, fl, a);
  else k1_flux<SCH_JS><<<nb, 128, 0, s>>>(c.g, q, fl, a);
  k1_rk<<<(c.g.n0 + 127) / 128, 128, 0, s>>>(c.g, fl, q4(c.du2), q, 1.0 / p.delta[0], dt, A, B, update);
  *launches += 2;
}

}  // namespace osb
