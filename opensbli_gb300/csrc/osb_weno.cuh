// osb_weno.cuh -- the per-interface arithmetic of the characteristic WENO5-JS flux, shared by the
// tiled and the line-marching flux kernels.
//
// Restates the generated "LLFWeno_reconstruction_d_direction" kernels (shock_capturing.py:146-155,
// 257-265) for one interface of a Cartesian block:
//   * Roe average at i+1/2 (schemes/spatial/averaging.py:70-114):
//       rho^ = sqrt(rho_L rho_R), u^ = (sqrt(rho_L) u_L + sqrt(rho_R) u_R)/(sqrt(rho_L)+sqrt(rho_R)),
//       H^ likewise from (p+rhoE)/rho, a^ = sqrt((gama-1)(H^ - |u^|^2/2));
//   * Euler eigensystem for the unit normal of direction d
//     (physical_models/euler_eigensystem.py:107-135): eigenvalues (u_d,u_d,u_d,u_d+a,u_d-a);
//   * LLF splitting (shock_capturing.py:357-398, 464-536): CF = LEV.F, CS = LEV.Q at i-2..i+3,
//     lambda_r = max over those six points of |ev_r| from the point values, f+- = CF +- lambda CS;
//   * WENO5-JS (weno.py:70-205, 341-369): the reference keeps the splitting's factor 1/2 out of f
//     and puts it into the smoothness indicators (1/4 of Jiang-Shu's) and the candidate stencils
//     (1/2 of the usual ones); alpha_r = d_r/(eps + beta_r)^2, omega_r = alpha_r / sum alpha;
//   * flux = REV.(fhat+ + fhat-) (shock_capturing.py:418-448).
//
// Arithmetic is rearranged for fewer instructions, not changed in meaning: sqrt(rho_L) u_L is formed
// as rhou_L / sqrt(rho_L); the three dense LEV rows (entropy and both acoustic waves) share one
// dot product g = (phi, -(g-1)u, g-1).X and h = X_{1+d} - u_d X_0 (the flux vector F is never
// stored: its projections are formed from Q, u_d and p):
//     acoustic+- . X = bt (g +- a h),   entropy . X = X_0 - g / a^2;
// the smoothness indicators use Jiang and Shu's sum-of-squares form built from first and second
// differences, and the candidates enter as p1 plus weighted third differences.  The nonlinear weights:
// in FP32 alpha_r = d_r * rcp((eps+beta_r)^2) with the fast hardware reciprocal (2 ulp), applied to
// the candidate differences (p_r - p_1) only; in FP64,
// where every division costs a Newton sequence on the slow FP64 pipe, the three alphas are scaled
// by the common factor prod_s (eps+beta_s)^2, alpha_0 ~ d_0 (eps+beta_1)^2 (eps+beta_2)^2 etc., so
// one exact division per side remains (the products stay far inside the FP64 range).  FP32 WENO-JS/Z
// run both sides of a characteristic reconstruction in the two lanes of the f32x2 instructions
// (weno5_pair12).
#pragma once
#include "osb_common.cuh"

namespace osb {

// sqrt(x) and 1/sqrt(x) of a positive x: FP32 from the hardware reciprocal square root (one SFU
// operation), FP64 from the correctly rounded square root and one exact division
__device__ __forceinline__ void sqrt_rsqrt(float x, float &s, float &is) {
  is = rsqrtf(x);
  s = x * is;
}
__device__ __forceinline__ void sqrt_rsqrt(double x, double &s, double &is) {
  s = sqrt(x);
  is = 1.0 / s;
}

// Schemes of the nonlinear weights
// (SCH_FILTER: the characteristic flux of the WENO5 non-linear filter, filter_flux)
enum { SCH_JS = 0, SCH_Z = 1, SCH_TENO = 2, SCH_TENO6 = 3, SCH_FILTER = 4 };

// One WENO5 side.  f0..f4 are the five stencil values ordered from the far upwind point to the
// far downwind one (for the right-going side: points i-2..i+2; for the left-going side the caller
// passes points i+3..i-1).  d0 weights the most downwind candidate (3/10), d2 the most upwind (1/10).
// JS: alpha_r = d_r / (eps + beta_r)^2.  Z (weno.py:283-331, Borges et al.): alpha_r =
// d_r (1 + (tau / (eps + beta_r))^2) with tau = |beta_0 - beta_2| (eps 1e-14 in the reference).
template <typename T, int SCH> __device__ __forceinline__ T weno5_side(T f0, T f1, T f2, T f3, T f4, T eps) {
  // first differences d_i = f_{i+1} - f_i; second differences t_r (the Jiang-Shu curvature terms);
  // s_r the one-sided slopes of each candidate stencil
  const T d0 = f1 - f0, d1 = f2 - f1, d2 = f3 - f2, d3 = f4 - f3;
  const T t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const T s0 = d3 - T(3) * d2, s1 = d1 + d2, s2 = T(3) * d1 - d0;
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T b0 = c13 * t0 * t0 + c14 * s0 * s0;
  const T b1 = c13 * t1 * t1 + c14 * s1 * s1;
  const T b2 = c13 * t2 * t2 + c14 * s2 * s2;
  const T e0 = b0 + eps, e1 = b1 + eps, e2 = b2 + eps;
  const T q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
  // candidates (with the reference's factor 1/2): p1 = f2/2 + d1/12 + d2/6, and the other two
  // through third differences, p0 - p1 = -(t0 - t1)/12, p2 - p1 = (t2 - t1)/6; the result
  // sum_r omega_r p_r = p1 + omega_0 (p0 - p1) + omega_2 (p2 - p1) scales only those differences by
  // the weights
  const T p1 = T(0.5) * f2 + T(1.0 / 12.0) * d1 + T(1.0 / 6.0) * d2;
  const T D0 = t0 - t1, D2 = t2 - t1;
  if (sizeof(T) == 8) {
    // alphas scaled by q0 q1 q2: one exact division per side
    T a0, a1, a2;
    if (SCH == SCH_Z) {
      const T tt = (b0 - b2) * (b0 - b2);
      a0 = T(3.0 / 10.0) * (q0 + tt) * (q1 * q2);
      a1 = T(3.0 / 5.0) * (q1 + tt) * (q0 * q2);
      a2 = T(1.0 / 10.0) * (q2 + tt) * (q0 * q1);
    } else {
      a0 = T(3.0 / 10.0) * (q1 * q2);
      a1 = T(3.0 / 5.0) * (q0 * q2);
      a2 = T(1.0 / 10.0) * (q0 * q1);
    }
    return p1 + (T(-1.0 / 12.0) * a0 * D0 + T(1.0 / 6.0) * a2 * D2) / (a0 + a1 + a2);
  } else {
    // fast hardware reciprocals: their rounding scales only the small third differences
    T a0, a1, a2;
    if (SCH == SCH_Z) {
      const T tt = (b0 - b2) * (b0 - b2);
      a0 = T(3.0 / 10.0) + T(3.0 / 10.0) * tt * rcp_t(q0);
      a1 = T(3.0 / 5.0) + T(3.0 / 5.0) * tt * rcp_t(q1);
      a2 = T(1.0 / 10.0) + T(1.0 / 10.0) * tt * rcp_t(q2);
    } else {
      a0 = T(3.0 / 10.0) * rcp_t(q0);
      a1 = T(3.0 / 5.0) * rcp_t(q1);
      a2 = T(1.0 / 10.0) * rcp_t(q2);
    }
    return p1 + (T(-1.0 / 12.0) * a0 * D0 + T(1.0 / 6.0) * a2 * D2) * rcp_t(a0 + a1 + a2);
  }
}

// ---- two-lane FP32: the f32x2 instructions of sm_100 and later run both sides of one characteristic
// reconstruction (+ side in the low lane, - side in the high lane) in one 64-bit register pair,
// halving the instructions of the side arithmetic.  Each lane rounds as the scalar instruction does.
struct F2 {
  unsigned long long v;
};
__device__ __forceinline__ F2 f2(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_split(F2 x, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x.v));
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a * b + c, one rounding per lane
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
__device__ __forceinline__ F2 rcp2(F2 x) {
  float a, b;
  f2_split(x, a, b);
  return f2(__fdividef(1.0f, a), __fdividef(1.0f, b));
}

// weno5_side (JS or Z) for both sides at once, FP32, returning 12x the reconstruction.  Rearranged
// for few instructions and few constant registers, the same quantities as weno5_side:
//   * indicators taken 16x (13/3 t^2 + s^2, with 16 eps): the weights depend on beta and eps only
//     through ratios, so the common factor cancels;
//   * alphas taken 10x: a = (3 r0, 6 r1, r2) with r = 1/(eps+beta)^2 (JS), a = (3 w0, 6 w1, w2) with
//     w = 1 + tau^2 r (Z), so 12 (p0 - p1) a0 / sum a = -3 r0 D0 / sum and 12 (p2 - p1) a2 / sum
//     = 2 r2 D2 / sum;
//   * 12 p1 = 6 f2 + d1 + 2 d2.
template <int SCH> __device__ __forceinline__ F2 weno5_pair12(F2 f0, F2 f1, F2 f2_, F2 f3, F2 f4, float eps) {
  const F2 m3 = f2(-3.0f, -3.0f), p3 = f2(3.0f, 3.0f), p6 = f2(6.0f, 6.0f);
  const F2 nd0 = f0 - f1, d1 = f2_ - f1, d2 = f3 - f2_, d3 = f4 - f3;
  const F2 t0 = d3 - d2, t1 = d2 - d1, t2 = d1 + nd0;
  const F2 s0 = fma2(m3, d2, d3), s1 = d1 + d2, s2 = fma2(p3, d1, nd0);
  const F2 k13 = f2(13.0f / 3.0f, 13.0f / 3.0f), e16 = f2(16.0f * eps, 16.0f * eps);
  const F2 e0 = fma2(k13 * t0, t0, s0 * s0) + e16;
  const F2 e1 = fma2(k13 * t1, t1, s1 * s1) + e16;
  const F2 e2 = fma2(k13 * t2, t2, s2 * s2) + e16;
  const F2 r0 = rcp2(e0 * e0), r1 = rcp2(e1 * e1), r2 = rcp2(e2 * e2);
  const F2 D0 = t0 - t1, D2 = t2 - t1;
  const F2 x = fma2(p6, f2_, s1 + d2);
  F2 w0, w2, sum;
  if constexpr (SCH == SCH_Z) {
    // the 16x indicators: tau and eps + beta carry the same factor
    const F2 bd = e0 - e2, tt = bd * bd, one = f2(1.0f, 1.0f);
    sum = fma2(tt, fma2(p3, r0, fma2(p6, r1, r2)), f2(10.0f, 10.0f));
    w0 = fma2(tt, r0, one);
    w2 = fma2(tt, r2, one);
  } else {
    sum = fma2(p3, r0, fma2(p6, r1, r2));
    w0 = r0;
    w2 = r2;
  }
  const F2 y = fma2(w2 + w2, D2, m3 * w0 * D0);
  return fma2(y, rcp2(sum), x);
}

// One TENO5 side with a fixed cut-off (schemes/spatial/teno.py:57-213, 407-465), the same stencil
// order as weno5_side.  The indicators of the halved values are weno5_side's b1 (central stencil),
// b0 (downwind) and b2 (upwind); tau = |beta_central - beta_upwind| (the reference's tau5 = |b0 - b2|
// in its own numbering); alpha_r = (1 + tau/(eps + beta_r))^6, formed as ratios to the largest base
// so that the sixth power cannot overflow; delta_r = 0 where alpha_r / sum alpha < ct; weights
// d = 11/20 (central), 2/5 (downwind), 1/20 (upwind), normalised over the kept candidates and applied
// to the candidate differences from the central one (as weno5_side does).
template <typename T> __device__ __forceinline__ T teno5_side(T f0, T f1, T f2, T f3, T f4, T eps, T ct) {
  const T d0 = f1 - f0, d1 = f2 - f1, d2 = f3 - f2, d3 = f4 - f3;
  const T t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const T s0 = d3 - T(3) * d2, s1 = d1 + d2, s2 = T(3) * d1 - d0;
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T bd = c13 * t0 * t0 + c14 * s0 * s0;  // downwind
  const T bc = c13 * t1 * t1 + c14 * s1 * s1;  // central
  const T bu = c13 * t2 * t2 + c14 * s2 * s2;  // upwind
  const T tau = abs_t(bc - bu);
  const T mc = T(1) + tau * rcp_t(eps + bc), md = T(1) + tau * rcp_t(eps + bd), mu = T(1) + tau * rcp_t(eps + bu);
  const T im = rcp_t(max_t(mc, max_t(md, mu)));
  const T nc = mc * im, nd = md * im, nu = mu * im;
  const T qc = (nc * nc) * (nc * nc) * (nc * nc), qd = (nd * nd) * (nd * nd) * (nd * nd),
          qu = (nu * nu) * (nu * nu) * (nu * nu);
  const T iq = rcp_t(qc + qd + qu);
  const T wc = ct > qc * iq ? T(0) : T(11.0 / 20.0);
  const T wd = ct > qd * iq ? T(0) : T(2.0 / 5.0);
  const T wu = ct > qu * iq ? T(0) : T(1.0 / 20.0);
  const T p1 = T(0.5) * f2 + T(1.0 / 12.0) * d1 + T(1.0 / 6.0) * d2;
  return p1 + (T(-1.0 / 12.0) * wd * (t0 - t1) + T(1.0 / 6.0) * wu * (t2 - t1)) * rcp_t(wc + wd + wu);
}

// One TENO6 side with a fixed cut-off (schemes/spatial/teno.py:94-192, 216-234, 407-465).  f0..f5
// run from the far upwind point to one past the far downwind one (+ side: points i-2..i+3; - side:
// i+3..i-2).  Candidates: the three TENO5 stencils and f2..f5; indicators of the halved values, the
// fourth one (f2..f5) as the reference generates it: 1/36 A^2 + 13/12 B^2 plus, on the + side, the linear
// third-difference term 781/720 C and on the - side 781/720 C^2 (teno.py:175-176 vs 183-185), with A, B,
// C its first-, second- and third-derivative combinations; tau6 = |b_c/6 - 2 b_d/3 + b_u/6 - b_4|;
// alpha_r = (1 + tau6/(eps + beta_r))^6 as ratios to the largest base (in magnitude: the + side's
// fourth indicator may be negative); weights 231/500, 3/10, 27/500, 23/125 for the central, downwind,
// upwind and four-point candidates, applied to candidate differences from the central one.
template <typename T>
__device__ __forceinline__ T teno6_side(T f0, T f1, T f2, T f3, T f4, T f5, bool plus, T eps, T ct) {
  const T d0 = f1 - f0, d1 = f2 - f1, d2 = f3 - f2, d3 = f4 - f3, d4 = f5 - f4;
  const T t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const T s0 = d3 - T(3) * d2, s1 = d1 + d2, s2 = T(3) * d1 - d0;
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T bd = c13 * t0 * t0 + c14 * s0 * s0;
  const T bc = c13 * t1 * t1 + c14 * s1 * s1;
  const T bu = c13 * t2 * t2 + c14 * s2 * s2;
  const T A = T(11) * d2 - T(7) * d3 + T(2) * d4, B = T(3) * d3 - T(2) * d2 - d4, C = d2 - T(2) * d3 + d4;
  const T b4 = T(1.0 / 144.0) * A * A + c13 * B * B + (plus ? T(781.0 / 1440.0) * C : T(781.0 / 2880.0) * C * C);
  const T tau = abs_t(T(1.0 / 6.0) * (bc + bu) - T(2.0 / 3.0) * bd - b4);
  const T mc = T(1) + tau * rcp_t(eps + bc), md = T(1) + tau * rcp_t(eps + bd), mu = T(1) + tau * rcp_t(eps + bu),
          m4 = T(1) + tau * rcp_t(eps + b4);
  const T im = rcp_t(max_t(max_t(abs_t(mc), abs_t(md)), max_t(abs_t(mu), abs_t(m4))));
  const T nc = mc * im, nd = md * im, nu = mu * im, n4 = m4 * im;
  const T qc = (nc * nc) * (nc * nc) * (nc * nc), qd = (nd * nd) * (nd * nd) * (nd * nd),
          qu = (nu * nu) * (nu * nu) * (nu * nu), q4 = (n4 * n4) * (n4 * n4) * (n4 * n4);
  const T iq = rcp_t((qc + qd) + (qu + q4));
  const T wc = ct > qc * iq ? T(0) : T(231.0 / 500.0);
  const T wd = ct > qd * iq ? T(0) : T(3.0 / 10.0);
  const T wu = ct > qu * iq ? T(0) : T(27.0 / 500.0);
  const T w4 = ct > q4 * iq ? T(0) : T(23.0 / 125.0);
  const T p1 = T(0.5) * f2 + T(1.0 / 12.0) * d1 + T(1.0 / 6.0) * d2;
  const T num = T(-1.0 / 12.0) * wd * (t0 - t1) + T(1.0 / 6.0) * wu * (t2 - t1) +
                T(1.0 / 24.0) * w4 * (T(5) * d2 - T(2) * d1 - T(4) * d3 + d4);
  return p1 + num * rcp_t((wc + wd) + (wu + w4));
}

// Per-point window entry: conserved vector Q, u_D, a, p.  The physical flux along D,
// F = (Q_{1+D}, Q_{1+c} u_D + delta_cD p, (p + Q_4) u_D), is folded into the projections below.
template <typename T> struct WPt {
  T Q[5], ud, a, p;
  // FP32 only: F(next point) - F(this point), each flux carried as a double-float sum (PtFlux), so
  // the difference is rounded once relative to its own size; FP64 leaves it unused
  T dF[5];
};

// FP32 physical flux of one point as an unevaluated sum h + l (double-float): h is the flux rounded
// to FP32, l what that rounding and the rounding of u_D and p discarded.  The characteristic
// projections act on flux differences between nearby points (O(delta)), so the FP32 rounding of
// each point's flux (O(1)) would otherwise enter them as noise of relative size 2^-24 / delta.
struct PtFlux {
  float h[5], l[5];
};

// The double-float flux (Q_{1+D}, Q_{1+c} u_D + delta_cD p, (Q_4 + p) u_D) from u_D and p as hi/lo
// pairs: products split by FMA (Dekker), sums by two-sum (Knuth).
template <int D>
__device__ __forceinline__ void point_flux_ff(const float (&r)[5], float ud, float ud_lo, float p, float p_lo,
                                              PtFlux &pf) {
  pf.h[0] = r[1 + D];
  pf.l[0] = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float m = r[1 + c];
    const float ph = __fmul_rn(m, ud);
    const float pl = fmaf(m, ud, -ph) + m * ud_lo;
    if (c == D) {
      const float sh = __fadd_rn(ph, p), bv = __fsub_rn(sh, ph);
      const float es = __fadd_rn(__fsub_rn(ph, __fsub_rn(sh, bv)), __fsub_rn(p, bv));
      pf.h[1 + c] = sh;
      pf.l[1 + c] = es + pl + p_lo;
    } else {
      pf.h[1 + c] = ph;
      pf.l[1 + c] = pl;
    }
  }
  const float sh = __fadd_rn(r[4], p), bv = __fsub_rn(sh, r[4]);
  const float es = __fadd_rn(__fsub_rn(r[4], __fsub_rn(sh, bv)), __fsub_rn(p, bv));
  const float h = __fmul_rn(sh, ud);
  pf.h[4] = h;
  pf.l[4] = fmaf(sh, ud, -h) + fmaf(es + p_lo, ud, sh * ud_lo);
}

// Primitive quantities of one point from its conserved vector.  1/rho is a correctly rounded
// division: the velocity enters the physical flux directly, and a biased reciprocal would bias
// every flux difference by the same relative amount, step after step.
// In FP32, u_D and p are rounded once from their exact values (prims_f32).
// With pf (FP32), also the point's double-float flux (point_flux_ff); lo2 (FP32, may be null)
// receives u_D's and p's remainders, for kernels that stage points and form the flux later.
template <typename T, int D>
__device__ __forceinline__ void point_prims(const T (&r)[5], T gm1, T gm1_lo, T gama, WPt<T> &w,
                                            PtFlux *pf = nullptr, float *lo2 = nullptr) {
  T irho, p;
  if constexpr (sizeof(T) == 4) {
    float u[3], p_lo;
    prims_f32(r[0], r[1], r[2], r[3], r[4], gm1, gm1_lo, irho, u, p, p_lo);
    w.ud = u[D];
    const float ud_lo = fmaf(-u[D], r[0], r[1 + D]) * irho;  // (m - u rho) exactly, over rho
    if (pf) point_flux_ff<D>(r, u[D], ud_lo, p, p_lo, *pf);
    if (lo2) {
      lo2[0] = ud_lo;
      lo2[1] = p_lo;
    }
  } else {
    irho = T(1) / r[0];
    const T u0 = r[1] * irho, u1 = r[2] * irho, u2 = r[3] * irho;
    p = gm1 * (r[4] - T(0.5) * (r[1] * u0 + r[2] * u1 + r[3] * u2));
    w.ud = D == 0 ? u0 : D == 1 ? u1 : u2;
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) w.Q[v] = r[v];
  w.p = p;
  T ia;
  sqrt_rsqrt(gama * p * irho, w.a, ia);
}

// FP32: record F(next) - F(prev) at the earlier of two consecutive points (rounded once)
__device__ __forceinline__ void link_flux(WPt<float> &prev, const PtFlux &fprev, const PtFlux &fnext) {
#pragma unroll
  for (int v = 0; v < 5; ++v) prev.dF[v] = __fsub_rn(fnext.h[v], fprev.h[v]) + __fsub_rn(fnext.l[v], fprev.l[v]);
}
__device__ __forceinline__ void link_flux(WPt<double> &, const PtFlux &, const PtFlux &) {}

// FP32: the same flux in difference form about window point 2 (point i).  The reconstruction
// reproduces constants (candidates are consistent, weights sum to one) and the splitting is linear,
// so replacing every point's conserved vector Q_t and physical flux F_t by Q_t - Q_i and F_t - F_i
// makes it return LEV.(F^ - F_i), and REV maps that to G = F_{i+1/2} - F_i (REV LEV = I).  The
// projections then act on differences of neighbouring points instead of O(1) values: their FP32
// rounding, which otherwise dominates the flux differences that form the residual, shrinks with the
// differences.  The flux differences F_t - F_i come from the window's consecutive-point differences
// dF (double-float point fluxes, rounded once per difference) by prefix sums.  Returns G: the caller
// forms F_{i+1/2} - F_{i-1/2} = (F_i - F_{i-1}) + (G_i - G_{i-1}) without ever rounding F_{i+1/2}.
template <int D, int SCH>
__device__ __forceinline__ void interface_flux_delta(const WPt<float> (&W)[6], const float gm1, const float igm1,
                                                     const float eps, const float ct, float out[5]) {
  using T = float;
  constexpr int E1 = (D + 1) % 3, E2 = (D + 2) % 3;
  constexpr int e1 = 3 - E1 - D, e2 = 3 - E2 - D;
  // ---- Roe average of points 2 and 3 (as below)
  const T rl = W[2].Q[0], rr = W[3].Q[0];
  T sl, sr, isl, isr;
  sqrt_rsqrt(rl, sl, isl);
  sqrt_rsqrt(rr, sr, isr);
  const T rho = sl * sr;
  const T inv_s = rcp_t(sl + sr);
  T u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = inv_s * (W[2].Q[1 + c] * isl + W[3].Q[1 + c] * isr);
  const T Hh = inv_s * ((W[2].p + W[2].Q[4]) * isl + (W[3].p + W[3].Q[4]) * isr);
  const T usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  T a, ia;
  sqrt_rsqrt(gm1 * (Hh - T(0.5) * usq), a, ia);
  const T irho = isl * isr;
  const T phi = gm1 * T(0.5) * usq;
  const T bt = T(0.70710678118654752440) * irho * ia;
  const T al = T(0.70710678118654752440) * rho * ia;
  const T ia2 = ia * ia;
  const T btA = bt * a;
  T lam_u = T(0), lam_p = T(0), lam_m = T(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    lam_u = max_t(lam_u, abs_t(W[t].ud));
    lam_p = max_t(lam_p, abs_t(W[t].ud + W[t].a));
    lam_m = max_t(lam_m, abs_t(W[t].a - W[t].ud));
  }
  auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
    if constexpr (SCH == SCH_JS || SCH == SCH_Z) {
      // + side f_k = cf[k] + lam cs[k] (points i-2..i+2), - side f_k = cf[5-k] - lam cs[5-k] (i+3..i-1)
      const F2 pm = f2(lam, -lam);
      F2 f[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) f[k] = fma2(pm, f2(cs[k], cs[5 - k]), f2(cf[k], cf[5 - k]));
      float rp, rm;
      f2_split(weno5_pair12<SCH>(f[0], f[1], f[2], f[3], f[4], eps), rp, rm);
      // 1/12 as an FP32 hi/lo pair: FP32 1/12 alone is 3e-8 high and would scale every reconstructed
      // flux the same way, a bias that grows in time
      constexpr float c12 = 1.0f / 12.0f, c12_lo = (float)(1.0 / 12.0 - (double)(1.0f / 12.0f));
      return mul_hl(rp + rm, c12, c12_lo);
    }
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    if constexpr (SCH == SCH_TENO6)
      return teno6_side<T>(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], true, eps, ct) +
             teno6_side<T>(fm[5], fm[4], fm[3], fm[2], fm[1], fm[0], false, eps, ct);
    else if constexpr (SCH == SCH_TENO)
      return teno5_side<T>(fp[0], fp[1], fp[2], fp[3], fp[4], eps, ct) +
             teno5_side<T>(fm[5], fm[4], fm[3], fm[2], fm[1], eps, ct);
    else
      return weno5_side<T, SCH>(fp[0], fp[1], fp[2], fp[3], fp[4], eps) +
             weno5_side<T, SCH>(fm[5], fm[4], fm[3], fm[2], fm[1], eps);
  };
  // F_t - F_i for the six window points from the consecutive differences
  T DF[6][5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    DF[2][v] = T(0);
    DF[3][v] = W[2].dF[v];
    DF[4][v] = W[2].dF[v] + W[3].dF[v];
    DF[5][v] = DF[4][v] + W[4].dF[v];
    DF[1][v] = -W[1].dF[v];
    DF[0][v] = -(W[1].dF[v] + W[0].dF[v]);
  }
  auto dQ = [&](int t, int v) -> T { return t == 2 ? T(0) : W[t].Q[v] - W[2].Q[v]; };
  auto dF = [&](int t, int v) -> T { return DF[t][v]; };

  const T se1 = (D == (E1 + 1) % 3) ? T(1) : T(-1), se2 = (D == (E2 + 1) % 3) ? T(1) : T(-1);
  T rE1, rE2;
  {
    T cf[6], cs[6];
    const T sr1 = se1 * irho;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = sr1 * (u[e1] * dF(t, 0) - dF(t, 1 + e1));
      cs[t] = sr1 * (u[e1] * dQ(t, 0) - dQ(t, 1 + e1));
    }
    rE1 = recon(cf, cs, lam_u);
    const T sr2 = se2 * irho;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = sr2 * (u[e2] * dF(t, 0) - dF(t, 1 + e2));
      cs[t] = sr2 * (u[e2] * dQ(t, 0) - dQ(t, 1 + e2));
    }
    rE2 = recon(cf, cs, lam_u);
  }
  T gQ[6], gF[6], hQ[6], hF[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const T uq = u[0] * dQ(t, 1) + u[1] * dQ(t, 2) + u[2] * dQ(t, 3);
    const T uf = u[0] * dF(t, 1) + u[1] * dF(t, 2) + u[2] * dF(t, 3);
    gQ[t] = phi * dQ(t, 0) - gm1 * uq + gm1 * dQ(t, 4);
    hQ[t] = dQ(t, 1 + D) - u[D] * dQ(t, 0);
    gF[t] = phi * dF(t, 0) - gm1 * uf + gm1 * dF(t, 4);
    hF[t] = dF(t, 1 + D) - u[D] * dF(t, 0);
  }
  T rD, r3, r4;
  {
    T cf[6], cs[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = dF(t, 0) - gF[t] * ia2;
      cs[t] = dQ(t, 0) - gQ[t] * ia2;
    }
    rD = recon(cf, cs, lam_u);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] + btA * hF[t];
      cs[t] = bt * gQ[t] + btA * hQ[t];
    }
    r3 = recon(cf, cs, lam_p);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] - btA * hF[t];
      cs[t] = bt * gQ[t] - btA * hQ[t];
    }
    r4 = recon(cf, cs, lam_m);
  }
  const T sac = r3 + r4, dac = r3 - r4;
  const T hh = (phi + a * a) * igm1;
  T G[5];
  G[0] = rD + al * sac;
#pragma unroll
  for (int c = 0; c < 3; ++c) G[1 + c] = u[c] * rD + al * (u[c] * sac + (c == D ? a * dac : T(0)));
  G[4] = (phi * igm1) * rD + al * (hh * sac + u[D] * a * dac);
  G[1 + e1] -= se1 * rho * rE1;
  G[4] -= se1 * rho * u[e1] * rE1;
  G[1 + e2] -= se2 * rho * rE2;
  G[4] -= se2 * rho * u[e2] * rE2;
#pragma unroll
  for (int v = 0; v < 5; ++v) out[v] = G[v];
}

// The characteristic flux about the averaged interface state (rho, u, a; irho = 1/rho, ia = 1/a):
// LEV/REV of the Euler eigensystem for the unit normal of direction D, CF = LEV.F and CS = LEV.Q at
// the six window points, the LLF wave speeds over the window, recon(cf, cs, lam) per characteristic,
// and REV back to conserved space.  Shared by the characteristic flux of the residual (Roe average,
// FP64 arithmetic) and by the WENO filter (simple average, both precisions).
template <typename T, int D, typename Recon>
__device__ __forceinline__ void char_flux(const WPt<T> (&W)[6], const T gm1, const T igm1, const T rho, const T irho,
                                          const T (&u)[3], const T a, const T ia, Recon recon, T out[5]) {
  constexpr int E1 = (D + 1) % 3, E2 = (D + 2) % 3;  // the two tangential axes (shear rows)
  constexpr int e1 = 3 - E1 - D, e2 = 3 - E2 - D;    // third axis of each shear row
  const T usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const T phi = gm1 * T(0.5) * usq;
  const T bt = T(0.70710678118654752440) * irho * ia;  // 1/(sqrt(2) rho a)
  const T al = T(0.70710678118654752440) * rho * ia;   // rho/(sqrt(2) a)
  const T ia2 = ia * ia;
  const T btA = bt * a;

  T lam_u = T(0), lam_p = T(0), lam_m = T(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    lam_u = max_t(lam_u, abs_t(W[t].ud));
    lam_p = max_t(lam_p, abs_t(W[t].ud + W[t].a));
    lam_m = max_t(lam_m, abs_t(W[t].a - W[t].ud));
  }

  // ---- shear rows: LEV_r . X = (s/rho)(u_e X_0 - X_{1+e}); for X = F: X_0 = Q_{1+D}, X_{1+e} = Q_{1+e} u_D
  const T se1 = (D == (E1 + 1) % 3) ? T(1) : T(-1), se2 = (D == (E2 + 1) % 3) ? T(1) : T(-1);
  T rE1, rE2;
  {
    T cf[6], cs[6];
    const T sr1 = se1 * irho;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = sr1 * (u[e1] * W[t].Q[1 + D] - W[t].Q[1 + e1] * W[t].ud);
      cs[t] = sr1 * (u[e1] * W[t].Q[0] - W[t].Q[1 + e1]);
    }
    rE1 = recon(cf, cs, lam_u);
    const T sr2 = se2 * irho;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = sr2 * (u[e2] * W[t].Q[1 + D] - W[t].Q[1 + e2] * W[t].ud);
      cs[t] = sr2 * (u[e2] * W[t].Q[0] - W[t].Q[1 + e2]);
    }
    rE2 = recon(cf, cs, lam_u);
  }
  // ---- dense rows share g = phi X_0 - (g-1) u.X_{1..3} + (g-1) X_4 and h = X_{1+D} - u_D X_0
  T gQ[6], gF[6], hQ[6], hF[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const WPt<T> &w = W[t];
    const T dq = u[0] * w.Q[1] + u[1] * w.Q[2] + u[2] * w.Q[3];
    gQ[t] = phi * w.Q[0] - gm1 * dq + gm1 * w.Q[4];
    hQ[t] = w.Q[1 + D] - u[D] * w.Q[0];
    gF[t] = phi * w.Q[1 + D] - gm1 * (w.ud * dq + u[D] * w.p) + gm1 * (w.p + w.Q[4]) * w.ud;
    hF[t] = w.Q[1 + D] * w.ud + w.p - u[D] * w.Q[1 + D];
  }
  T rD, r3, r4;
  {
    T cf[6], cs[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = W[t].Q[1 + D] - gF[t] * ia2;
      cs[t] = W[t].Q[0] - gQ[t] * ia2;
    }
    rD = recon(cf, cs, lam_u);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] + btA * hF[t];
      cs[t] = bt * gQ[t] + btA * hQ[t];
    }
    r3 = recon(cf, cs, lam_p);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      cf[t] = bt * gF[t] - btA * hF[t];
      cs[t] = bt * gQ[t] - btA * hQ[t];
    }
    r4 = recon(cf, cs, lam_m);
  }

  // ---- back to conserved space: flux = REV . rec
  const T sac = r3 + r4, dac = r3 - r4;
  const T hh = (phi + a * a) * igm1;
  out[0] = rD + al * sac;
#pragma unroll
  for (int c = 0; c < 3; ++c) out[1 + c] = u[c] * rD + al * (u[c] * sac + (c == D ? a * dac : T(0)));
  out[4] = (phi * igm1) * rD + al * (hh * sac + u[D] * a * dac);
  // shear columns: REV[1+e][r] = -s rho, REV[4][r] = -s rho u_e
  out[1 + e1] -= se1 * rho * rE1;
  out[4] -= se1 * rho * u[e1] * rE1;
  out[1 + e2] -= se2 * rho * rE2;
  out[4] -= se2 * rho * u[e2] * rE2;
}

// WENO5-JS side (weno5_side) that also reports the filter's weight sensor of that side,
// sum_r |omega_r / d_r - 1|^4 / (9^4 + 2) (schemes/spatial/weno.py:436-452, sensor_theta = 4; d_r the
// optimal weights, so 1/min(d) - 1 = 9)
template <typename T> __device__ __forceinline__ T weno5_side_sensor(T f0, T f1, T f2, T f3, T f4, T eps, T &sens) {
  const T d0 = f1 - f0, d1 = f2 - f1, d2 = f3 - f2, d3 = f4 - f3;
  const T t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const T s0 = d3 - T(3) * d2, s1 = d1 + d2, s2 = T(3) * d1 - d0;
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T e0 = c13 * t0 * t0 + c14 * s0 * s0 + eps;
  const T e1 = c13 * t1 * t1 + c14 * s1 * s1 + eps;
  const T e2 = c13 * t2 * t2 + c14 * s2 * s2 + eps;
  const T q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
  // alphas over the common factor q0 q1 q2 (one division)
  const T a0 = T(3.0 / 10.0) * (q1 * q2), a1 = T(3.0 / 5.0) * (q0 * q2), a2 = T(1.0 / 10.0) * (q0 * q1);
  const T is = T(1) / (a0 + a1 + a2);
  const T w0 = a0 * is, w1 = a1 * is, w2 = a2 * is;
  const T x0 = T(10.0 / 3.0) * w0 - T(1), x1 = T(5.0 / 3.0) * w1 - T(1), x2 = T(10) * w2 - T(1);
  sens = ((x0 * x0) * (x0 * x0) + (x1 * x1) * (x1 * x1) + (x2 * x2) * (x2 * x2)) * T(1.0 / 6563.0);
  const T p1 = T(0.5) * f2 + T(1.0 / 12.0) * d1 + T(1.0 / 6.0) * d2;
  return p1 + (T(-1.0 / 12.0) * w0 * (t0 - t1) + T(1.0 / 6.0) * w2 * (t2 - t1));
}

// Interface flux of the WENO5 non-linear filter (filters/WENO_filter.py:15-339 with the LLF WENO5-JS
// scheme it builds, schemes/spatial/weno.py:474-483): the characteristic flux about the simple average
// of rho, u and a over points i, i+1 (averaging.py SimpleAverage([0, 1])), whose reconstructed
// characteristics are replaced by rj (Recon - central) with rj the larger of the two sides' weight
// sensors and central = (CF_{i-2} - 8 CF_{i-1} + 37 CF_i + 37 CF_{i+1} - 8 CF_{i+2} + CF_{i+3}) / 60,
// the 6th-order central interpolation of the characteristic fluxes (shock_capturing.py:399-412, 440-442).
template <typename T, int D>
__device__ __forceinline__ void filter_flux(const WPt<T> (&W)[6], const T gm1, const T igm1, T out[5]) {
  const T eps = T(1e-6);  // the filter's LLFWeno is WENO-JS, whose epsilon is 1e-6 (weno.py:341-369)
  const T rho = T(0.5) * (W[3].Q[0] + W[2].Q[0]);
  const T ir2 = T(1) / W[2].Q[0], ir3 = T(1) / W[3].Q[0];
  T u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = T(0.5) * (W[3].Q[1 + c] * ir3 + W[2].Q[1 + c] * ir2);
  const T a = T(0.5) * (W[2].a + W[3].a);
  const T ia = T(1) / a, irho = T(1) / rho;
  auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    T sp, sm;
    const T rec = weno5_side_sensor<T>(fp[0], fp[1], fp[2], fp[3], fp[4], eps, sp) +
                  weno5_side_sensor<T>(fm[5], fm[4], fm[3], fm[2], fm[1], eps, sm);
    const T central = T(1.0 / 60.0) * ((cf[0] + cf[5]) - T(8) * (cf[1] + cf[4]) + T(37) * (cf[2] + cf[3]));
    return max_t(sp, sm) * (rec - central);
  };
  char_flux<T, D>(W, gm1, igm1, rho, irho, u, a, ia, recon, out);
}

// Characteristic flux at the interface between window points 2 and 3 (points i and i+1), and for
// SCH_FILTER the WENO filter's flux there.  ct: the TENO cut-off (unused by the other schemes).
// FP64 and the filter: out = F_{i+1/2}.  Other FP32 schemes: out = G = F_{i+1/2} - F_i
// (interface_flux_delta); flux_difference below turns either into the cell's F_{i+1/2} - F_{i-1/2}.
template <typename T, int D, int SCH>
__device__ __forceinline__ void interface_flux(const WPt<T> (&W)[6], const T gm1, const T igm1, const T eps,
                                               const T ct, T out[5]) {
  if constexpr (SCH == SCH_FILTER) {
    filter_flux<T, D>(W, gm1, igm1, out);
  } else if constexpr (sizeof(T) == 4) {
    interface_flux_delta<D, SCH>(W, gm1, igm1, eps, ct, out);
  } else {
    // ---- Roe average of points 2 and 3
    const T rl = W[2].Q[0], rr = W[3].Q[0];
    T sl, sr, isl, isr;  // sqrt(rho) and 1/sqrt(rho) of both sides
    sqrt_rsqrt(rl, sl, isl);
    sqrt_rsqrt(rr, sr, isr);
    const T rho = sl * sr;
    const T inv_s = rcp_t(sl + sr);
    T u[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c] = inv_s * (W[2].Q[1 + c] * isl + W[3].Q[1 + c] * isr);
    const T Hh = inv_s * ((W[2].p + W[2].Q[4]) * isl + (W[3].p + W[3].Q[4]) * isr);
    const T usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    T a, ia;
    sqrt_rsqrt(gm1 * (Hh - T(0.5) * usq), a, ia);
    const T irho = isl * isr;
    auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
      T fp[6], fm[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        fp[t] = cf[t] + lam * cs[t];
        fm[t] = cf[t] - lam * cs[t];
      }
      if constexpr (SCH == SCH_TENO6)
        return teno6_side<T>(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], true, eps, ct) +
               teno6_side<T>(fm[5], fm[4], fm[3], fm[2], fm[1], fm[0], false, eps, ct);
      else if constexpr (SCH == SCH_TENO)
        return teno5_side<T>(fp[0], fp[1], fp[2], fp[3], fp[4], eps, ct) +
               teno5_side<T>(fm[5], fm[4], fm[3], fm[2], fm[1], eps, ct);
      else
        return weno5_side<T, SCH>(fp[0], fp[1], fp[2], fp[3], fp[4], eps) +
               weno5_side<T, SCH>(fm[5], fm[4], fm[3], fm[2], fm[1], eps);
    };
    char_flux<T, D>(W, gm1, igm1, rho, irho, u, a, ia, recon, out);
  }
}

// F_{i+1/2} - F_{i-1/2} of variable v for the cell whose left interface flux (or its G) was `prev`
// and right one `cur`; W is the window of the right interface (W[1], W[2] = points i-1, i).
// (FP32 residual fluxes come as G; the filter's fluxes, and all FP64 ones, as the full flux)
template <int SCH> __device__ __forceinline__ float flux_difference(const WPt<float> (&W)[6], int v, float cur, float prev) {
  if constexpr (SCH == SCH_FILTER) return cur - prev;
  else return W[1].dF[v] + (cur - prev);
}
template <int SCH>
__device__ __forceinline__ double flux_difference(const WPt<double> (&)[6], int, double cur, double prev) {
  return cur - prev;
}

}  // namespace osb
