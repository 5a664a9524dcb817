// osb_adjoint_weno.cuh -- reverse mode of the FP64 characteristic WENO5-JS interface flux
// (osb_weno.cuh::interface_flux, FP64 branch, with point_prims): given the adjoint F_bar of the flux
// F_{i+1/2}, the contributions (dF/dQ_t)^T F_bar to the six conserved vectors of its window.
//
// The forward quantities are recomputed in the same order and then swept backwards.  The LLF wave
// speeds are maxima over the window: their derivative goes to the first point attaining the maximum
// (the forward keeps the earlier of equal values), with the sign of the absolute value.  WENO5-JS
// weights are smooth, so the nonlinear weights are differentiated exactly.
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

// one WENO5-JS side (weno5_side<double, SCH_JS>): forward value
OSB_ADJ_HD double side(const double f[5], double eps) {
  const double d0 = f[1] - f[0], d1 = f[2] - f[1], d2 = f[3] - f[2], d3 = f[4] - f[3];
  const double t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const double s0 = d3 - 3.0 * d2, s1 = d1 + d2, s2 = 3.0 * d1 - d0;
  const double c13 = 13.0 / 48.0, c14 = 1.0 / 16.0;
  const double e0 = c13 * t0 * t0 + c14 * s0 * s0 + eps, e1 = c13 * t1 * t1 + c14 * s1 * s1 + eps,
               e2 = c13 * t2 * t2 + c14 * s2 * s2 + eps;
  const double q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
  const double a0 = 0.3 * q1 * q2, a1 = 0.6 * q0 * q2, a2 = 0.1 * q0 * q1;
  const double p1 = 0.5 * f[2] + d1 / 12.0 + d2 / 6.0;
  return p1 + (-a0 * (t0 - t1) / 12.0 + a2 * (t2 - t1) / 6.0) / (a0 + a1 + a2);
}

// its reverse: fb[k] += d(side)/df_k * yb
OSB_ADJ_HD void side_adj(const double f[5], double yb, double eps, double fb[5]) {
  const double d0 = f[1] - f[0], d1 = f[2] - f[1], d2 = f[3] - f[2], d3 = f[4] - f[3];
  const double t0 = d3 - d2, t1 = d2 - d1, t2 = d1 - d0;
  const double s0 = d3 - 3.0 * d2, s1 = d1 + d2, s2 = 3.0 * d1 - d0;
  const double c13 = 13.0 / 48.0, c14 = 1.0 / 16.0;
  const double e0 = c13 * t0 * t0 + c14 * s0 * s0 + eps, e1 = c13 * t1 * t1 + c14 * s1 * s1 + eps,
               e2 = c13 * t2 * t2 + c14 * s2 * s2 + eps;
  const double q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
  const double a0 = 0.3 * q1 * q2, a1 = 0.6 * q0 * q2, a2 = 0.1 * q0 * q1;
  const double D0 = t0 - t1, D2 = t2 - t1;
  const double iS = 1.0 / (a0 + a1 + a2);
  const double N = -a0 * D0 / 12.0 + a2 * D2 / 6.0;
  const double Nb = yb * iS, Sb = -yb * N * iS * iS;
  const double a0b = Nb * (-D0 / 12.0) + Sb, a2b = Nb * (D2 / 6.0) + Sb, a1b = Sb;
  const double D0b = Nb * (-a0 / 12.0), D2b = Nb * (a2 / 6.0);
  const double q0b = a1b * 0.6 * q2 + a2b * 0.1 * q1;
  const double q1b = a0b * 0.3 * q2 + a2b * 0.1 * q0;
  const double q2b = a0b * 0.3 * q1 + a1b * 0.6 * q0;
  const double b0b = 2.0 * e0 * q0b, b1b = 2.0 * e1 * q1b, b2b = 2.0 * e2 * q2b;
  const double t0b = 2.0 * c13 * t0 * b0b + D0b, s0b = 2.0 * c14 * s0 * b0b;
  const double t1b = 2.0 * c13 * t1 * b1b - D0b - D2b, s1b = 2.0 * c14 * s1 * b1b;
  const double t2b = 2.0 * c13 * t2 * b2b + D2b, s2b = 2.0 * c14 * s2 * b2b;
  const double d3b = s0b + t0b;
  const double d2b = yb / 6.0 - 3.0 * s0b + s1b - t0b + t1b;
  const double d1b = yb / 12.0 + s1b + 3.0 * s2b - t1b + t2b;
  const double d0b = -s2b - t2b;
  fb[0] -= d0b;
  fb[1] += d0b - d1b;
  fb[2] += d1b - d2b + 0.5 * yb;
  fb[3] += d2b - d3b;
  fb[4] += d3b;
}

// one characteristic row: forward reconstruction of f+- = cf +- lam cs, both sides
OSB_ADJ_HD double recon(const double cf[6], const double cs[6], double lam, double eps) {
  double fp[5], fm[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    fp[t] = cf[t] + lam * cs[t];
    fm[t] = cf[5 - t] - lam * cs[5 - t];
  }
  return side(fp, eps) + side(fm, eps);
}

// its reverse: cfb, csb (6 points) and lamb accumulated
OSB_ADJ_HD void recon_adj(const double cf[6], const double cs[6], double lam, double yb, double eps,
                                          double cfb[6], double csb[6], double &lamb) {
  double fp[5], fm[5], fpb[5] = {0, 0, 0, 0, 0}, fmb[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    fp[t] = cf[t] + lam * cs[t];
    fm[t] = cf[5 - t] - lam * cs[5 - t];
  }
  side_adj(fp, yb, eps, fpb);
  side_adj(fm, yb, eps, fmb);
#pragma unroll
  for (int t = 0; t < 5; ++t) {
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
template <int D>
OSB_ADJ_HD void interface_flux_adj(const double (&Q)[6][5], const double (&Fb)[5], double gama,
                                            double (&Qb)[6][5], double *F = nullptr, double eps = EPS_JS) {
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
  const double rE1 = recon(cfE1, csE1, lu, eps), rE2 = recon(cfE2, csE2, lu, eps);
  const double rD = recon(cfD, csD, lu, eps), r3 = recon(cf3, cs3, lp, eps), r4 = recon(cf4, cs4, lm, eps);
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
  recon_adj(cf4, cs4, lm, r4b, eps, cf4b, cs4b, lmb);
  recon_adj(cf3, cs3, lp, r3b, eps, cf3b, cs3b, lpb);
  recon_adj(cfD, csD, lu, rDb, eps, cfDb, csDb, lub);
  recon_adj(cfE1, csE1, lu, rE1b, eps, cfE1b, csE1b, lub);
  recon_adj(cfE2, csE2, lu, rE2b, eps, cfE2b, csE2b, lub);
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
