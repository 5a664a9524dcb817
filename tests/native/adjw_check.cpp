// Checks the reverse mode of the FP64 characteristic WENO5-JS interface flux
// (opensbli_gb300/csrc/osb_adjoint_weno.cuh) against central finite differences of its own forward
// flux, for all three directions on random smooth windows and windows with a jump.  Prints the
// worst relative error and the number of windows checked.
#include <math.h>
#include <stdio.h>

#include <random>

#include "osb_adjoint_weno.cuh"

template <int D> static double check(std::mt19937_64 &rng, bool jump) {
  std::normal_distribution<double> N(0.0, 1.0);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const double g = 1.4;
  double Q[6][5];
  const double r0 = 1.0 + 0.2 * U(rng), p0 = 0.5 + 0.1 * U(rng);
  double u0[3] = {0.5 * N(rng), 0.5 * N(rng), 0.5 * N(rng)};
  for (int t = 0; t < 6; ++t) {
    const double j = (jump && t >= 3) ? 0.5 : 0.0;
    const double r = r0 + j + 0.05 * N(rng), p = p0 + 0.5 * j + 0.02 * N(rng);
    double u[3], ke = 0;
    for (int c = 0; c < 3; ++c) {
      u[c] = u0[c] + 0.1 * N(rng);
      ke += u[c] * u[c];
    }
    Q[t][0] = r;
    for (int c = 0; c < 3; ++c) Q[t][1 + c] = r * u[c];
    Q[t][4] = p / (g - 1) + 0.5 * r * ke;
  }
  double Fb[5];
  for (int v = 0; v < 5; ++v) Fb[v] = N(rng);
  double Qb[6][5] = {};
  osb::adjw::interface_flux_adj<D>(Q, Fb, g, Qb);
  double worst = 0, scale = 0;
  const double h = 1e-6;
  double fd[6][5];
  for (int t = 0; t < 6; ++t)
    for (int v = 0; v < 5; ++v) {
      double Qp[6][5], Qm[6][5], Fp[5], Fm[5], dummy[6][5] = {};
      const double z[5] = {0, 0, 0, 0, 0};
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 5; ++b) Qp[a][b] = Qm[a][b] = Q[a][b];
      Qp[t][v] += h;
      Qm[t][v] -= h;
      osb::adjw::interface_flux_adj<D>(Qp, z, g, dummy, Fp);
      osb::adjw::interface_flux_adj<D>(Qm, z, g, dummy, Fm);
      double s = 0;
      for (int k = 0; k < 5; ++k) s += (Fp[k] - Fm[k]) * Fb[k];
      fd[t][v] = s / (2 * h);
      scale = fmax(scale, fabs(fd[t][v]));
    }
  for (int t = 0; t < 6; ++t)
    for (int v = 0; v < 5; ++v) worst = fmax(worst, fabs(fd[t][v] - Qb[t][v]));
  return worst / scale;
}

int main() {
  std::mt19937_64 rng(7);
  double worst = 0;
  int n = 0;
  for (int k = 0; k < 300; ++k) {
    const bool jump = k % 4 == 3;
    worst = fmax(worst, check<0>(rng, jump));
    worst = fmax(worst, check<1>(rng, jump));
    worst = fmax(worst, check<2>(rng, jump));
    n += 3;
  }
  printf("%.3e %d\n", worst, n);
  return 0;
}
