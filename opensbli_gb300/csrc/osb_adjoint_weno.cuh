// osb_adjoint_weno.cuh -- reverse mode of the FP64 characteristic interface flux
// (osb_weno.cuh::interface_flux, FP64 branch, with point_prims) for WENO5-JS, WENO5-Z, TENO5 and
// TENO6: given the adjoint F_bar of the flux F_{i+1/2}, the contributions (dF/dQ_t)^T F_bar to the six
// conserved vectors of its window.
//
// The forward quantities are recomputed in the same order and then swept backwards.  The LLF wave
// speeds are maxima over the window: their derivative goes to the first point attaining the maximum
// (the forward keeps the earlier of equal values), with the sign of the absolute value.  The WENO
// weights are smooth and differentiated exactly; the TENO cut-off is a step function of the
// indicators, so between switches the TENO weights are constants and only the candidates vary.
// Plain C++ apart from the qualifiers, so the host compiler can check it against finite differences.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define OSB_ADJ_HD __host__ __device__ inline
#else
#define OSB_ADJ_HD inline
#endif

namespace osb {
namespace adjw {

constexpr double EPS_JS = 1e-6;

// Schemes, numbered as the flux kernels number them: WENO5-JS, WENO5-Z, TENO5, TENO6.
enum { ADJ_JS = 0, ADJ_Z = 1, ADJ_TENO5 = 2, ADJ_TENO6 = 3 };

// The nonlinear weights of one side as the FP64 flux kernels form them (osb_weno.cuh: weno5_side,
// teno5_side, teno6_side).  f[0..5] run from the far upwind point to one past the far downwind one;
// the 5-point schemes use f[0..4].  Returns the reconstruction; w[0..3] receive the weights of the
// candidate differences (see below) and W their normaliser, so that
//   y = p1 + (w[0] (-(t0 - t1)/12) + w[1] ((t2 - t1)/6) + w[2] ((-2 d1 + 5 d2 - 4 d3 + d4)/24)) / W.
// WENO: w = (a0, a2, 0) and W = a0 + a1 + a2 depend smoothly on f; TENO: w and W are the cut-off's
// selections of the optimal weights, constant between switches.
template <int SCH>
OSB_ADJ_HD double side_weights(const double f[6], bool plus, double eps, double ct, double w[3], double &W) {
  const double d0 = f[1] - f[0], d1 = f[2] - f[1], d2 = f[3] - f[2], d3 = f[4] - f[3];
  const double t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const double s0 = d3 - 3.0 * d2, s1 = d1 + d2, s2 = 3.0 * d1 - d0;
  const double c13 = 13.0 / 48.0, c14 = 1.0 / 16.0;
  const double b0 = c13 * t0 * t0 + c14 * s0 * s0, b1 = c13 * t1 * t1 + c14 * s1 * s1,
               b2 = c13 * t2 * t2 + c14 * s2 * s2;
  w[2] = 0.0;
  if (SCH == ADJ_JS || SCH == ADJ_Z) {
    const double q0 = (b0 + eps) * (b0 + eps), q1 = (b1 + eps) * (b1 + eps), q2 = (b2 + eps) * (b2 + eps);
    const double tt = SCH == ADJ_Z ? (b0 - b2) * (b0 - b2) : 0.0;
    const double a0 = SCH == ADJ_Z ? 0.3 * (q0 + tt) * (q1 * q2) : 0.3 * q1 * q2;
    const double a1 = SCH == ADJ_Z ? 0.6 * (q1 + tt) * (q0 * q2) : 0.6 * q0 * q2;
    const double a2 = SCH == ADJ_Z ? 0.1 * (q2 + tt) * (q0 * q1) : 0.1 * q0 * q1;
    w[0] = a0;
    w[1] = a2;
    W = a0 + a1 + a2;
  } else {
    // TENO: indicators central b1, downwind b0, upwind b2 (+ the four-point one for TENO6)
    double m[4], tau;
    int nr = 3;
    double b4 = 0.0;
    if (SCH == ADJ_TENO6) {
      const double d4 = f[5] - f[4];
      const double A = 11.0 * d2 - 7.0 * d3 + 2.0 * d4, B = 3.0 * d3 - 2.0 * d2 - d4, C = d2 - 2.0 * d3 + d4;
      b4 = (1.0 / 144.0) * A * A + c13 * B * B + (plus ? (781.0 / 1440.0) * C : (781.0 / 2880.0) * C * C);
      tau = fabs((1.0 / 6.0) * (b1 + b2) - (2.0 / 3.0) * b0 - b4);
      nr = 4;
    } else {
      tau = fabs(b1 - b2);
    }
    const double bb[4] = {b1, b0, b2, b4};  // central, downwind, upwind, four-point
    double mm = 0.0;
    for (int r = 0; r < nr; ++r) {
      m[r] = 1.0 + tau * (1.0 / (eps + bb[r]));
      mm = fmax(mm, fabs(m[r]));
    }
    const double im = 1.0 / mm;
    double q[4], qs = 0.0;
    for (int r = 0; r < nr; ++r) {
      const double n = m[r] * im;
      q[r] = (n * n) * (n * n) * (n * n);
    }
    qs = nr == 4 ? (q[0] + q[1]) + (q[2] + q[3]) : q[0] + q[1] + q[2];
    const double iq = 1.0 / qs;
    const double dw5[3] = {11.0 / 20.0, 2.0 / 5.0, 1.0 / 20.0}, dw6[4] = {231.0 / 500.0, 3.0 / 10.0, 27.0 / 500.0, 23.0 / 125.0};
    double wr[4];
    for (int r = 0; r < nr; ++r) wr[r] = ct > q[r] * iq ? 0.0 : (nr == 4 ? dw6[r] : dw5[r]);
    w[0] = wr[1];  // downwind
    w[1] = wr[2];  // upwind
    w[2] = nr == 4 ? wr[3] : 0.0;
    W = nr == 4 ? (wr[0] + wr[1]) + (wr[2] + wr[3]) : wr[0] + wr[1] + wr[2];
  }
  const double p1 = 0.5 * f[2] + d1 / 12.0 + d2 / 6.0;
  const double c3 = SCH == ADJ_TENO6 ? (5.0 * d2 - 2.0 * d1 - 4.0 * d3 + (f[5] - f[4])) / 24.0 : 0.0;
  return p1 + (w[0] * (-(t0 - t1) / 12.0) + w[1] * ((t2 - t1) / 6.0) + w[2] * c3) / W;
}

template <int SCH> OSB_ADJ_HD double side(const double f[6], bool plus, double eps, double ct) {
  double w[3], W;
  return side_weights<SCH>(f, plus, eps, ct, w, W);
}

// reverse of one side: fb[k] += d(side)/df_k * yb (TENO weights held at their selection)
template <int SCH>
OSB_ADJ_HD void side_adj(const double f[6], bool plus, double yb, double eps, double ct, double fb[6]) {
  const double d0 = f[1] - f[0], d1 = f[2] - f[1], d2 = f[3] - f[2], d3 = f[4] - f[3];
  const double t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const double D0 = t0 - t1, D2 = t2 - t1;
  const double d4 = SCH == ADJ_TENO6 ? f[5] - f[4] : 0.0;
  double w[3], W;
  side_weights<SCH>(f, plus, eps, ct, w, W);
  const double c3 = SCH == ADJ_TENO6 ? (5.0 * d2 - 2.0 * d1 - 4.0 * d3 + d4) / 24.0 : 0.0;
  const double iW = 1.0 / W;
  const double N = w[0] * (-D0 / 12.0) + w[1] * (D2 / 6.0) + w[2] * c3;
  // y = p1 + N / W
  double D0b = yb * iW * (-w[0] / 12.0), D2b = yb * iW * (w[1] / 6.0);
  const double c3b = yb * iW * w[2];
  double t0b = D0b, t1b = -D0b - D2b, t2b = D2b;
  double d0b = 0, d1b = yb / 12.0, d2b = yb / 6.0, d3b = 0, d4b = 0;
  d1b += -2.0 / 24.0 * c3b;
  d2b += 5.0 / 24.0 * c3b;
  d3b += -4.0 / 24.0 * c3b;
  d4b += 1.0 / 24.0 * c3b;
  if (SCH == ADJ_JS || SCH == ADJ_Z) {
    // smooth weights: w0 = a0, w1 = a2, W = a0 + a1 + a2
    const double s0 = d3 - 3.0 * d2, s1 = d1 + d2, s2 = 3.0 * d1 - d0;
    const double c13 = 13.0 / 48.0, c14 = 1.0 / 16.0;
    const double b0 = c13 * t0 * t0 + c14 * s0 * s0, b1 = c13 * t1 * t1 + c14 * s1 * s1,
                 b2 = c13 * t2 * t2 + c14 * s2 * s2;
    const double e0 = b0 + eps, e1 = b1 + eps, e2 = b2 + eps;
    const double q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
    const double Wb = -yb * N * iW * iW;
    const double a0b = yb * iW * (-D0 / 12.0) + Wb, a2b = yb * iW * (D2 / 6.0) + Wb, a1b = Wb;
    double q0b, q1b, q2b, b0b = 0, b2b = 0;
    if (SCH == ADJ_Z) {
      const double tt = (b0 - b2) * (b0 - b2);
      // a0 = 0.3 (q0 + tt) q1 q2, a1 = 0.6 (q1 + tt) q0 q2, a2 = 0.1 (q2 + tt) q0 q1
      q0b = a0b * 0.3 * q1 * q2 + a1b * 0.6 * (q1 + tt) * q2 + a2b * 0.1 * (q2 + tt) * q1;
      q1b = a0b * 0.3 * (q0 + tt) * q2 + a1b * 0.6 * q0 * q2 + a2b * 0.1 * (q2 + tt) * q0;
      q2b = a0b * 0.3 * (q0 + tt) * q1 + a1b * 0.6 * (q1 + tt) * q0 + a2b * 0.1 * q0 * q1;
      const double ttb = a0b * 0.3 * q1 * q2 + a1b * 0.6 * q0 * q2 + a2b * 0.1 * q0 * q1;
      b0b += 2.0 * (b0 - b2) * ttb;
      b2b -= 2.0 * (b0 - b2) * ttb;
    } else {
      q0b = a1b * 0.6 * q2 + a2b * 0.1 * q1;
      q1b = a0b * 0.3 * q2 + a2b * 0.1 * q0;
      q2b = a0b * 0.3 * q1 + a1b * 0.6 * q0;
    }
    b0b += 2.0 * e0 * q0b;
    const double b1b = 2.0 * e1 * q1b;
    b2b += 2.0 * e2 * q2b;
    t0b += 2.0 * c13 * t0 * b0b;
    t1b += 2.0 * c13 * t1 * b1b;
    t2b += 2.0 * c13 * t2 * b2b;
    const double s0b = 2.0 * c14 * s0 * b0b, s1b = 2.0 * c14 * s1 * b1b, s2b = 2.0 * c14 * s2 * b2b;
    d3b += s0b;
    d2b += -3.0 * s0b + s1b;
    d1b += s1b + 3.0 * s2b;
    d0b += -s2b;
  }
  // t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0
  d3b += t0b;
  d2b += -t0b + t1b;
  d1b += -t1b + t2b;
  d0b += -t2b;
  fb[0] -= d0b;
  fb[1] += d0b - d1b;
  fb[2] += d1b - d2b + 0.5 * yb;
  fb[3] += d2b - d3b;
  fb[4] += d3b - d4b;
  fb[5] += d4b;
}

// one characteristic row: the + side on f+ = cf + lam cs at points 0..5, the - side on
// f- = cf - lam cs at points 5..0
template <int SCH>
OSB_ADJ_HD double recon(const double cf[6], const double cs[6], double lam, double eps, double ct) {
  double fp[6], fm[6];
  for (int t = 0; t < 6; ++t) {
    fp[t] = cf[t] + lam * cs[t];
    fm[t] = cf[5 - t] - lam * cs[5 - t];
  }
  return side<SCH>(fp, true, eps, ct) + side<SCH>(fm, false, eps, ct);
}

// its reverse: cfb, csb (6 points) and lamb accumulated
template <int SCH>
OSB_ADJ_HD void recon_adj(const double cf[6], const double cs[6], double lam, double yb, double eps, double ct,
                          double cfb[6], double csb[6], double &lamb) {
  double fp[6], fm[6], fpb[6] = {0, 0, 0, 0, 0, 0}, fmb[6] = {0, 0, 0, 0, 0, 0};
  for (int t = 0; t < 6; ++t) {
    fp[t] = cf[t] + lam * cs[t];
    fm[t] = cf[5 - t] - lam * cs[5 - t];
  }
  side_adj<SCH>(fp, true, yb, eps, ct, fpb);
  side_adj<SCH>(fm, false, yb, eps, ct, fmb);
  for (int t = 0; t < 6; ++t) {
    cfb[t] += fpb[t];
    csb[t] += lam * fpb[t];
    lamb += cs[t] * fpb[t];
    cfb[5 - t] += fmb[t];
    csb[5 - t] -= lam * fmb[t];
    lamb -= cs[5 - t] * fmb[t];
  }
}

// Q[t][v]: conserved vectors of window points i-2 .. i+3 (interface between 2 and 3); Fb: adjoint of
// the interface flux; Qb[t][v] += (dF/dQ_t)^T Fb.  F, if given, receives the forward flux.
template <int D, int SCH = ADJ_JS>
OSB_ADJ_HD void interface_flux_adj(const double (&Q)[6][5], const double (&Fb)[5], double gama,
                                            double (&Qb)[6][5], double *F = nullptr, double eps = EPS_JS,
                                            double ct = 0.0) {
  constexpr int E1 = (D + 1) % 3, E2 = (D + 2) % 3;
  constexpr int e1 = 3 - E1 - D, e2 = 3 - E2 - D;
  const double gm1 = gama - 1.0, igm1 = 1.0 / gm1, S2 = 0.70710678118654752440;
  // ---- point primitives
  double irt[6], uu[6][3], p[6], ud[6], at[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    irt[t] = 1.0 / Q[t][0];
#pragma unroll
    for (int c = 0; c < 3; ++c) uu[t][c] = Q[t][1 + c] * irt[t];
    p[t] = gm1 * (Q[t][4] - 0.5 * (Q[t][1] * uu[t][0] + Q[t][2] * uu[t][1] + Q[t][3] * uu[t][2]));
    ud[t] = uu[t][D];
    at[t] = sqrt(gama * p[t] * irt[t]);
  }
  // ---- Roe average of points 2 and 3
  const double sl = sqrt(Q[2][0]), sr = sqrt(Q[3][0]), isl = 1.0 / sl, isr = 1.0 / sr;
  const double rho = sl * sr, ssum = sl + sr, inv_s = 1.0 / ssum;
  double mu_[3], u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    mu_[c] = Q[2][1 + c] * isl + Q[3][1 + c] * isr;
    u[c] = inv_s * mu_[c];
  }
  const double mH = (p[2] + Q[2][4]) * isl + (p[3] + Q[3][4]) * isr;
  const double Hh = inv_s * mH;
  const double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double a = sqrt(gm1 * (Hh - 0.5 * usq)), ia = 1.0 / a;
  const double irho = isl * isr, phi = gm1 * 0.5 * usq;
  const double bt = S2 * irho * ia, al = S2 * rho * ia, ia2 = ia * ia, btA = bt * a;
  // ---- wave speeds (first maximum)
  int ku = 0, kp = 0, km = 0;
#pragma unroll
  for (int t = 1; t < 6; ++t) {
    if (fabs(ud[t]) > fabs(ud[ku])) ku = t;
    if (fabs(ud[t] + at[t]) > fabs(ud[kp] + at[kp])) kp = t;
    if (fabs(at[t] - ud[t]) > fabs(at[km] - ud[km])) km = t;
  }
  const double lu = fabs(ud[ku]), lp = fabs(ud[kp] + at[kp]), lm = fabs(at[km] - ud[km]);
  const double se1 = (D == (E1 + 1) % 3) ? 1.0 : -1.0, se2 = (D == (E2 + 1) % 3) ? 1.0 : -1.0;
  const double sr1 = se1 * irho, sr2 = se2 * irho;
  // ---- rows
  double cfE1[6], csE1[6], cfE2[6], csE2[6], dq[6], gQ[6], hQ[6], gF[6], hF[6];
  double cfD[6], csD[6], cf3[6], cs3[6], cf4[6], cs4[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    cfE1[t] = sr1 * (u[e1] * Q[t][1 + D] - Q[t][1 + e1] * ud[t]);
    csE1[t] = sr1 * (u[e1] * Q[t][0] - Q[t][1 + e1]);
    cfE2[t] = sr2 * (u[e2] * Q[t][1 + D] - Q[t][1 + e2] * ud[t]);
    csE2[t] = sr2 * (u[e2] * Q[t][0] - Q[t][1 + e2]);
    dq[t] = Q[t][1] * u[0] + Q[t][2] * u[1] + Q[t][3] * u[2];
    gQ[t] = phi * Q[t][0] - gm1 * dq[t] + gm1 * Q[t][4];
    hQ[t] = Q[t][1 + D] - u[D] * Q[t][0];
    gF[t] = phi * Q[t][1 + D] - gm1 * (ud[t] * dq[t] + u[D] * p[t]) + gm1 * (p[t] + Q[t][4]) * ud[t];
    hF[t] = Q[t][1 + D] * ud[t] + p[t] - u[D] * Q[t][1 + D];
    cfD[t] = Q[t][1 + D] - gF[t] * ia2;
    csD[t] = Q[t][0] - gQ[t] * ia2;
    cf3[t] = bt * gF[t] + btA * hF[t];
    cs3[t] = bt * gQ[t] + btA * hQ[t];
    cf4[t] = bt * gF[t] - btA * hF[t];
    cs4[t] = bt * gQ[t] - btA * hQ[t];
  }
  const double rE1 = recon<SCH>(cfE1, csE1, lu, eps, ct), rE2 = recon<SCH>(cfE2, csE2, lu, eps, ct);
  const double rD = recon<SCH>(cfD, csD, lu, eps, ct), r3 = recon<SCH>(cf3, cs3, lp, eps, ct),
               r4 = recon<SCH>(cf4, cs4, lm, eps, ct);
  const double sac = r3 + r4, dac = r3 - r4, hh = (phi + a * a) * igm1;
  if (F) {
    F[0] = rD + al * sac;
    for (int c = 0; c < 3; ++c) F[1 + c] = u[c] * rD + al * (u[c] * sac + (c == D ? a * dac : 0.0));
    F[4] = (phi * igm1) * rD + al * (hh * sac + u[D] * a * dac);
    F[1 + e1] -= se1 * rho * rE1;
    F[4] -= se1 * rho * u[e1] * rE1;
    F[1 + e2] -= se2 * rho * rE2;
    F[4] -= se2 * rho * u[e2] * rE2;
  }

  // ---- reverse: back-projection
  double ub[3] = {0, 0, 0};
  double rhob = 0, rE1b = 0, rE2b = 0, rDb = 0, alb = 0, phib = 0, ab = 0, hhb = 0, sacb = 0, dacb = 0;
  rhob += -se2 * rE2 * Fb[1 + e2] - se2 * u[e2] * rE2 * Fb[4];
  rE2b += -se2 * rho * Fb[1 + e2] - se2 * rho * u[e2] * Fb[4];
  ub[e2] += -se2 * rho * rE2 * Fb[4];
  rhob += -se1 * rE1 * Fb[1 + e1] - se1 * u[e1] * rE1 * Fb[4];
  rE1b += -se1 * rho * Fb[1 + e1] - se1 * rho * u[e1] * Fb[4];
  ub[e1] += -se1 * rho * rE1 * Fb[4];
  phib += igm1 * rD * Fb[4];
  rDb += phi * igm1 * Fb[4];
  alb += (hh * sac + u[D] * a * dac) * Fb[4];
  hhb += al * sac * Fb[4];
  sacb += al * hh * Fb[4];
  ub[D] += al * a * dac * Fb[4];
  ab += al * u[D] * dac * Fb[4];
  dacb += al * u[D] * a * Fb[4];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    ub[c] += (rD + al * sac) * Fb[1 + c];
    rDb += u[c] * Fb[1 + c];
    alb += (u[c] * sac + (c == D ? a * dac : 0.0)) * Fb[1 + c];
    sacb += al * u[c] * Fb[1 + c];
    if (c == D) {
      ab += al * dac * Fb[1 + c];
      dacb += al * a * Fb[1 + c];
    }
  }
  rDb += Fb[0];
  alb += sac * Fb[0];
  sacb += al * Fb[0];
  phib += igm1 * hhb;
  ab += 2.0 * a * igm1 * hhb;
  const double r3b = sacb + dacb, r4b = sacb - dacb;
  // ---- reverse: reconstructions
  double cfE1b[6] = {}, csE1b[6] = {}, cfE2b[6] = {}, csE2b[6] = {}, cfDb[6] = {}, csDb[6] = {};
  double cf3b[6] = {}, cs3b[6] = {}, cf4b[6] = {}, cs4b[6] = {};
  double lub = 0, lpb = 0, lmb = 0;
  recon_adj<SCH>(cf4, cs4, lm, r4b, eps, ct, cf4b, cs4b, lmb);
  recon_adj<SCH>(cf3, cs3, lp, r3b, eps, ct, cf3b, cs3b, lpb);
  recon_adj<SCH>(cfD, csD, lu, rDb, eps, ct, cfDb, csDb, lub);
  recon_adj<SCH>(cfE1, csE1, lu, rE1b, eps, ct, cfE1b, csE1b, lub);
  recon_adj<SCH>(cfE2, csE2, lu, rE2b, eps, ct, cfE2b, csE2b, lub);
  // ---- reverse: projections
  double btb = 0, btAb = 0, ia2b = 0, srb1 = 0, srb2 = 0;
  double udb[6] = {}, pb[6] = {}, atb[6] = {};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const double gFb = bt * (cf3b[t] + cf4b[t]) - ia2 * cfDb[t];
    const double hFb = btA * (cf3b[t] - cf4b[t]);
    const double gQb = bt * (cs3b[t] + cs4b[t]) - ia2 * csDb[t];
    const double hQb = btA * (cs3b[t] - cs4b[t]);
    btb += gF[t] * (cf3b[t] + cf4b[t]) + gQ[t] * (cs3b[t] + cs4b[t]);
    btAb += hF[t] * (cf3b[t] - cf4b[t]) + hQ[t] * (cs3b[t] - cs4b[t]);
    ia2b -= gF[t] * cfDb[t] + gQ[t] * csDb[t];
    Qb[t][1 + D] += cfDb[t];
    Qb[t][0] += csDb[t];
    // hF = Q[1+D] ud + p - u[D] Q[1+D]
    Qb[t][1 + D] += hFb * (ud[t] - u[D]);
    udb[t] += hFb * Q[t][1 + D];
    pb[t] += hFb;
    ub[D] -= hFb * Q[t][1 + D];
    // gF = phi Q[1+D] - gm1 (ud dq + u[D] p) + gm1 (p + Q4) ud
    phib += gFb * Q[t][1 + D];
    Qb[t][1 + D] += gFb * phi;
    udb[t] += gFb * (-gm1 * dq[t] + gm1 * (p[t] + Q[t][4]));
    double dqb = -gm1 * ud[t] * gFb;
    ub[D] -= gm1 * p[t] * gFb;
    pb[t] += gFb * gm1 * (ud[t] - u[D]);
    Qb[t][4] += gFb * gm1 * ud[t];
    // hQ = Q[1+D] - u[D] Q0
    Qb[t][1 + D] += hQb;
    Qb[t][0] -= u[D] * hQb;
    ub[D] -= hQb * Q[t][0];
    // gQ = phi Q0 - gm1 dq + gm1 Q4
    phib += gQb * Q[t][0];
    Qb[t][0] += phi * gQb;
    dqb -= gm1 * gQb;
    Qb[t][4] += gm1 * gQb;
    // dq = Q[1..3] . u
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Qb[t][1 + c] += dqb * u[c];
      ub[c] += Q[t][1 + c] * dqb;
    }
    // shear rows
    ub[e1] += sr1 * (cfE1b[t] * Q[t][1 + D] + csE1b[t] * Q[t][0]);
    Qb[t][1 + D] += sr1 * u[e1] * cfE1b[t];
    Qb[t][1 + e1] -= sr1 * (ud[t] * cfE1b[t] + csE1b[t]);
    udb[t] -= sr1 * Q[t][1 + e1] * cfE1b[t];
    Qb[t][0] += sr1 * u[e1] * csE1b[t];
    srb1 += cfE1b[t] * (u[e1] * Q[t][1 + D] - Q[t][1 + e1] * ud[t]) + csE1b[t] * (u[e1] * Q[t][0] - Q[t][1 + e1]);
    ub[e2] += sr2 * (cfE2b[t] * Q[t][1 + D] + csE2b[t] * Q[t][0]);
    Qb[t][1 + D] += sr2 * u[e2] * cfE2b[t];
    Qb[t][1 + e2] -= sr2 * (ud[t] * cfE2b[t] + csE2b[t]);
    udb[t] -= sr2 * Q[t][1 + e2] * cfE2b[t];
    Qb[t][0] += sr2 * u[e2] * csE2b[t];
    srb2 += cfE2b[t] * (u[e2] * Q[t][1 + D] - Q[t][1 + e2] * ud[t]) + csE2b[t] * (u[e2] * Q[t][0] - Q[t][1 + e2]);
  }
  double irhob = se1 * srb1 + se2 * srb2;
  // wave speeds; d|x|/dx is taken as 0 at x = 0 (where the wave speed vanishes on a whole window, as
  // on the Taylor-Green symmetry planes, the central difference of the forward is 0 there too)
  auto sgn = [](double x) { return x > 0 ? 1.0 : x < 0 ? -1.0 : 0.0; };
  udb[ku] += sgn(ud[ku]) * lub;
  {
    const double sp = sgn(ud[kp] + at[kp]);
    udb[kp] += sp * lpb;
    atb[kp] += sp * lpb;
    const double sm = sgn(at[km] - ud[km]);
    atb[km] += sm * lmb;
    udb[km] -= sm * lmb;
  }
  // Roe average constants
  btb += btAb * a;
  ab += btAb * bt;
  const double iab = S2 * irho * btb + S2 * rho * alb + 2.0 * ia * ia2b;
  irhob += S2 * ia * btb;
  rhob += S2 * ia * alb;
  double usqb = gm1 * 0.5 * phib;
  ab -= iab / (a * a);
  const double A2b = ab / (2.0 * a);
  const double Hhb = gm1 * A2b;
  usqb -= 0.5 * gm1 * A2b;
#pragma unroll
  for (int c = 0; c < 3; ++c) ub[c] += 2.0 * u[c] * usqb;
  double islb = isr * irhob, isrb = isl * irhob;
  double inv_sb = mH * Hhb;
#pragma unroll
  for (int c = 0; c < 3; ++c) inv_sb += mu_[c] * ub[c];
  const double mHb = inv_s * Hhb;
  pb[2] += isl * mHb;
  Qb[2][4] += isl * mHb;
  islb += (p[2] + Q[2][4]) * mHb;
  pb[3] += isr * mHb;
  Qb[3][4] += isr * mHb;
  isrb += (p[3] + Q[3][4]) * mHb;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double mub = inv_s * ub[c];
    Qb[2][1 + c] += isl * mub;
    islb += Q[2][1 + c] * mub;
    Qb[3][1 + c] += isr * mub;
    isrb += Q[3][1 + c] * mub;
  }
  const double ssumb = -inv_sb / (ssum * ssum);
  const double slb = ssumb + sr * rhob - islb / (sl * sl);
  const double srbb = ssumb + sl * rhob - isrb / (sr * sr);
  Qb[2][0] += slb / (2.0 * sl);
  Qb[3][0] += srbb / (2.0 * sr);
  // point primitives
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const double Atb = atb[t] / (2.0 * at[t]);
    pb[t] += gama * irt[t] * Atb;
    double irtb = gama * p[t] * Atb;
    double uub[3] = {0, 0, 0};
    uub[D] += udb[t];
    Qb[t][4] += gm1 * pb[t];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Qb[t][1 + c] += -0.5 * gm1 * pb[t] * uu[t][c];
      uub[c] += -0.5 * gm1 * pb[t] * Q[t][1 + c];
      Qb[t][1 + c] += uub[c] * irt[t];
      irtb += uub[c] * Q[t][1 + c];
    }
    Qb[t][0] -= irtb * irt[t] * irt[t];
  }
}

}  // namespace adjw
}  // namespace osb
