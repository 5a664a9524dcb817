// osb_weno.cu -- characteristic WENO5-JS flux kernels, one per direction.
//
// Restates the generated "LLFWeno_reconstruction_d_direction" kernels (shock_capturing.py:146-155,
// 257-265) and the "LLFWeno Residual" kernel (shock_capturing.py:21-34,
// opensblifunctions.py:575-593) for a Cartesian block, fused so that interface fluxes never reach
// HBM:
//   * Roe average at i+1/2 (schemes/spatial/averaging.py:70-114):
//       rho^ = sqrt(rho_L rho_R), u^ = (sqrt(rho_L) u_L + sqrt(rho_R) u_R)/(sqrt(rho_L)+sqrt(rho_R)),
//       H^ likewise from (p+rhoE)/rho, a^ = sqrt((gama-1)(H^ - |u^|^2/2));
//   * Euler eigensystem for the unit normal of direction d
//     (physical_models/euler_eigensystem.py:107-135): eigenvalues (u_d,u_d,u_d,u_d+a,u_d-a);
//   * LLF splitting (shock_capturing.py:357-398, 464-536): CF = LEV.F, CS = LEV.Q at i-2..i+3,
//     lambda_r = max over those six points of |ev_r| from the point values, f+- = CF +- lambda CS;
//   * WENO5-JS (weno.py:70-205, 341-369) in the reference's own form: smoothness indicators and
//     candidate stencils carry the splitting's factor 1/2, alpha_r = d_r/(eps + beta_r)^2;
//   * flux = REV.(fhat+ + fhat-) (shock_capturing.py:418-448);
//   * residual R -= (flux_{i+1/2} - flux_{i-1/2}) / delta_d.
//
// Tiling: a block covers TA lines along d and computes TI consecutive interfaces per line, giving
// the flux difference of TI-1 cells.  The primitive fields of the TI+5 points of every line sit in
// shared memory (loaded once, coalesced along x); each thread owns whole interfaces, keeps the six
// stencil points' conserved and flux vectors in registers and projects them one characteristic
// field at a time.
#include "osb_common.cuh"
#include "osb_internal.h"

namespace osb {

namespace {
enum { W_RHO = 0, W_RU0, W_RU1, W_RU2, W_E, W_P, W_A, W_UD, W_NF };

template <int DIR> struct WTile;
template <> struct WTile<0> {  // x: 64 interfaces x 4 rows, one interface per thread
  static constexpr int TI = 64, TA = 4, IPT = 1;
};
template <> struct WTile<1> {  // y: 32 x-lanes x 32 interfaces, four interfaces per thread
  static constexpr int TI = 32, TA = 32, IPT = 4;
};
template <> struct WTile<2> {
  static constexpr int TI = 32, TA = 32, IPT = 4;
};
}  // namespace

// WENO5-JS on f = CF + lambda CS at points i-2..i+2 (upwind side of i+1/2), reference form.
template <typename T> __device__ __forceinline__ T weno_plus(T f0, T f1, T f2, T f3, T f4, T eps) {
  const T h = T(0.5);
  const T b0 = h * f2 * (T(5.0 / 3.0) * f2 - T(31.0 / 6.0) * f3 + T(11.0 / 6.0) * f4) +
               h * f3 * (T(25.0 / 6.0) * f3 - T(19.0 / 6.0) * f4) + T(1.0 / 3.0) * f4 * f4;
  const T b1 = h * f1 * (T(2.0 / 3.0) * f1 - T(13.0 / 6.0) * f2 + T(5.0 / 6.0) * f3) +
               h * f2 * (T(13.0 / 6.0) * f2 - T(13.0 / 6.0) * f3) + T(1.0 / 3.0) * f3 * f3;
  const T b2 = h * f0 * (T(2.0 / 3.0) * f0 + T(11.0 / 6.0) * f2) +
               h * f1 * (T(-19.0 / 6.0) * f0 + T(25.0 / 6.0) * f1 - T(31.0 / 6.0) * f2) + T(5.0 / 6.0) * f2 * f2;
  const T a0 = T(3.0 / 10.0) / ((b0 + eps) * (b0 + eps));
  const T a1 = T(3.0 / 5.0) / ((b1 + eps) * (b1 + eps));
  const T a2 = T(1.0 / 10.0) / ((b2 + eps) * (b2 + eps));
  const T inv = T(1) / (a0 + a1 + a2);
  return a0 * inv * (T(1.0 / 6.0) * f2 + T(5.0 / 12.0) * f3 - T(1.0 / 12.0) * f4) +
         a1 * inv * (T(-1.0 / 12.0) * f1 + T(5.0 / 12.0) * f2 + T(1.0 / 6.0) * f3) +
         a2 * inv * (T(1.0 / 6.0) * f0 - T(7.0 / 12.0) * f1 + T(11.0 / 12.0) * f2);
}
// f = CF - lambda CS at points i-1..i+3 (f1..f5), reconstruct at i+1/2 from the right.
template <typename T> __device__ __forceinline__ T weno_minus(T f1, T f2, T f3, T f4, T f5, T eps) {
  const T h = T(0.5);
  const T b0 = h * f3 * (T(5.0 / 3.0) * f3 - T(31.0 / 6.0) * f4 + T(11.0 / 6.0) * f5) +
               h * f4 * (T(25.0 / 6.0) * f4 - T(19.0 / 6.0) * f5) + T(1.0 / 3.0) * f5 * f5;
  const T b1 = h * f2 * (T(2.0 / 3.0) * f2 - T(13.0 / 6.0) * f3 + T(5.0 / 6.0) * f4) +
               h * f3 * (T(13.0 / 6.0) * f3 - T(13.0 / 6.0) * f4) + T(1.0 / 3.0) * f4 * f4;
  const T b2 = h * f1 * (T(2.0 / 3.0) * f1 - T(19.0 / 6.0) * f2 + T(11.0 / 6.0) * f3) +
               h * f2 * (T(25.0 / 6.0) * f2 - T(31.0 / 6.0) * f3) + T(5.0 / 6.0) * f3 * f3;
  const T a0 = T(1.0 / 10.0) / ((b0 + eps) * (b0 + eps));
  const T a1 = T(3.0 / 5.0) / ((b1 + eps) * (b1 + eps));
  const T a2 = T(3.0 / 10.0) / ((b2 + eps) * (b2 + eps));
  const T inv = T(1) / (a0 + a1 + a2);
  return a0 * inv * (T(11.0 / 12.0) * f3 - T(7.0 / 12.0) * f4 + T(1.0 / 6.0) * f5) +
         a1 * inv * (T(1.0 / 6.0) * f2 + T(5.0 / 12.0) * f3 - T(1.0 / 12.0) * f4) +
         a2 * inv * (T(-1.0 / 12.0) * f1 + T(5.0 / 12.0) * f2 + T(1.0 / 6.0) * f3);
}

// Characteristic flux at one interface.  P(f, t) reads field f of stencil point t = 0..5 (points
// i-2..i+3); returns the five components of the interface flux.
template <typename T, int D, typename Pt>
__device__ __forceinline__ void interface_flux(const Pt &P, const T gama, const T eps, T out[5]) {
  constexpr int E1 = (D + 1) % 3, E2 = (D + 2) % 3;  // the two tangential axes
  const T gm1 = gama - T(1);
  // ---- Roe average of points 2 (i) and 3 (i+1)
  const T rl = P(W_RHO, 2), rr = P(W_RHO, 3);
  const T sl = sqrt_t(rl), sr = sqrt_t(rr);
  const T rho = sqrt_t(rl * rr);
  const T inv_s = T(1) / (sl + sr);
  T u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = inv_s * (sl * (P(W_RU0 + c, 2) / rl) + sr * (P(W_RU0 + c, 3) / rr));
  const T Hh = inv_s * ((P(W_P, 2) + P(W_E, 2)) / sl + (P(W_P, 3) + P(W_E, 3)) / sr);
  const T usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const T a = sqrt_t(gm1 * (Hh - T(0.5) * usq));
  const T ia = T(1) / a, irho = T(1) / rho;
  const T ia2 = ia * ia;
  const T phi = gm1 * T(0.5) * usq;
  const T bt = T(0.70710678118654752440) * irho * ia;  // 1/(sqrt(2) rho a)
  const T al = T(0.70710678118654752440) * rho * ia;   // rho/(sqrt(2) a)

  // ---- stencil vectors in registers
  T Q[6][5], F[6][5];
  T lam_u = T(0), lam_p = T(0), lam_m = T(0);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const T ud = P(W_UD, t), p = P(W_P, t), at = P(W_A, t);
    Q[t][0] = P(W_RHO, t);
    Q[t][1] = P(W_RU0, t);
    Q[t][2] = P(W_RU1, t);
    Q[t][3] = P(W_RU2, t);
    Q[t][4] = P(W_E, t);
    F[t][0] = Q[t][1 + D];
#pragma unroll
    for (int c = 0; c < 3; ++c) F[t][1 + c] = Q[t][1 + c] * ud + (c == D ? p : T(0));
    F[t][4] = (p + Q[t][4]) * ud;
    lam_u = max_t(lam_u, abs_t(ud));
    lam_p = max_t(lam_p, abs_t(ud + at));
    lam_m = max_t(lam_m, abs_t(at - ud));
  }

  T rec[5];
  // ---- row D: entropy wave, LEV_D = (1 - phi/a^2, (g-1)u_c/a^2, -(g-1)/a^2)
  {
    const T l0 = T(1) - phi * ia2, l1 = gm1 * u[0] * ia2, l2 = gm1 * u[1] * ia2, l3 = gm1 * u[2] * ia2,
            l4 = -gm1 * ia2;
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const T cf = l0 * F[t][0] + l1 * F[t][1] + l2 * F[t][2] + l3 * F[t][3] + l4 * F[t][4];
      const T cs = l0 * Q[t][0] + l1 * Q[t][1] + l2 * Q[t][2] + l3 * Q[t][3] + l4 * Q[t][4];
      fp[t] = cf + lam_u * cs;
      fm[t] = cf - lam_u * cs;
    }
    rec[D] = weno_plus(fp[0], fp[1], fp[2], fp[3], fp[4], eps) + weno_minus(fm[1], fm[2], fm[3], fm[4], fm[5], eps);
  }
  // ---- rows E1, E2: shear waves.  Row r (r != D), third axis e = 3 - r - D:
  //      LEV_r = (s u_e/rho) e_0 - (s/rho) e_{1+e}, s = +1 if D == (r+1)%3 else -1
#pragma unroll
  for (int w = 0; w < 2; ++w) {
    const int r = w == 0 ? E1 : E2;
    const int e = 3 - r - D;
    const T s = (D == (r + 1) % 3) ? T(1) : T(-1);
    const T l0 = s * u[e] * irho, le = -s * irho;
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const T cf = l0 * F[t][0] + le * F[t][1 + e];
      const T cs = l0 * Q[t][0] + le * Q[t][1 + e];
      fp[t] = cf + lam_u * cs;
      fm[t] = cf - lam_u * cs;
    }
    rec[r] = weno_plus(fp[0], fp[1], fp[2], fp[3], fp[4], eps) + weno_minus(fm[1], fm[2], fm[3], fm[4], fm[5], eps);
  }
  // ---- rows 3, 4: acoustic waves u_d + a, u_d - a
#pragma unroll
  for (int w = 0; w < 2; ++w) {
    const T sg = w == 0 ? T(-1) : T(1);  // row 3: phi - u_d a ; row 4: phi + u_d a
    const T lam = w == 0 ? lam_p : lam_m;
    T l[5];
    l[0] = bt * (phi + sg * u[D] * a);
#pragma unroll
    for (int c = 0; c < 3; ++c) l[1 + c] = -bt * (gm1 * u[c] + (c == D ? sg * a : T(0)));
    l[4] = bt * gm1;
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const T cf = l[0] * F[t][0] + l[1] * F[t][1] + l[2] * F[t][2] + l[3] * F[t][3] + l[4] * F[t][4];
      const T cs = l[0] * Q[t][0] + l[1] * Q[t][1] + l[2] * Q[t][2] + l[3] * Q[t][3] + l[4] * Q[t][4];
      fp[t] = cf + lam * cs;
      fm[t] = cf - lam * cs;
    }
    rec[3 + w] = weno_plus(fp[0], fp[1], fp[2], fp[3], fp[4], eps) + weno_minus(fm[1], fm[2], fm[3], fm[4], fm[5], eps);
  }
  // ---- back to conserved space: flux = REV . rec
  const T sac = rec[3] + rec[4], dac = rec[3] - rec[4];
  const T hh = (phi + a * a) / gm1;
  out[0] = rec[D] + al * sac;
#pragma unroll
  for (int c = 0; c < 3; ++c) out[1 + c] = u[c] * rec[D] + al * (u[c] * sac + (c == D ? a * dac : T(0)));
  out[4] = (phi / gm1) * rec[D] + al * (hh * sac + u[D] * a * dac);
  // shear columns: REV[1+e][r] = -s rho, REV[4][r] = -s rho u_e
#pragma unroll
  for (int w = 0; w < 2; ++w) {
    const int r = w == 0 ? E1 : E2;
    const int e = 3 - r - D;
    const T s = (D == (r + 1) % 3) ? T(1) : T(-1);
    out[1 + e] += -s * rho * rec[r];
    out[4] += -s * rho * u[e] * rec[r];
  }
}

template <typename T, int DIR, bool ACCUM>
__global__ void __launch_bounds__(256) k_weno(Grid g, Fields5<const T> q, Fields5<T> res, Phys ph) {
  using Tl = WTile<DIR>;
  constexpr int TI = Tl::TI, TA = Tl::TA, NPT = TI + 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sf = reinterpret_cast<T *>(smem_raw);   // [W_NF][NPT][TA] (DIR>0) or [W_NF][TA][NPT] (DIR==0)
  T *sflux = sf + W_NF * NPT * TA;           // [5][TI][TA] or [5][TA][TI]
  const int tid = threadIdx.x;
  const int n[3] = {g.n0, g.n1, g.n2};
  const T gm1 = T(ph.gama - 1.0), gama = T(ph.gama);
  const T eps = T(ph.weno_eps);

  // tile origin: first cell whose flux difference this block writes (d0), across-line origin
  int d0, a0, o1, o2;  // o1/o2: the remaining coordinates
  if (DIR == 0) { d0 = blockIdx.x * (TI - 1); a0 = blockIdx.y * TA; o2 = blockIdx.z; o1 = 0; }
  else if (DIR == 1) { a0 = blockIdx.x * TA; d0 = blockIdx.y * (TI - 1); o2 = blockIdx.z; o1 = 0; }
  else { a0 = blockIdx.x * TA; o1 = blockIdx.y; d0 = blockIdx.z * (TI - 1); o2 = 0; }

  auto sidx = [&](int f, int pos, int a) -> int {
    return DIR == 0 ? (f * TA + a) * NPT + pos : (f * NPT + pos) * TA + a;
  };
  auto coords = [&](int pos, int a, int &i, int &j, int &k) {
    const int c = d0 - 3 + pos;
    if (DIR == 0) { i = c; j = a0 + a; k = o2; }
    else if (DIR == 1) { i = a0 + a; j = c; k = o2; }
    else { i = a0 + a; j = o1; k = c; }
  };
  const int nd = n[DIR];
  const int na = DIR == 0 ? n[1] : n[0];

  // ---- load primitives of the tile's points
  for (int t = tid; t < NPT * TA; t += 256) {
    int pos, a;
    if (DIR == 0) { a = t / NPT; pos = t % NPT; }
    else { pos = t / TA; a = t % TA; }
    const int c = d0 - 3 + pos;
    if (c > nd + 2 || a0 + a >= na) continue;
    int i, j, k;
    coords(pos, a, i, j, k);
    const int64_t m = gidx(g, i, j, k);
    const T rho = q.v[0][m], r0 = q.v[1][m], r1 = q.v[2][m], r2 = q.v[3][m], E = q.v[4][m];
    const T u0 = r0 / rho, u1 = r1 / rho, u2 = r2 / rho;
    const T half = T(0.5);
    const T p = gm1 * (E - half * rho * u0 * u0 - half * rho * u1 * u1 - half * rho * u2 * u2);
    sf[sidx(W_RHO, pos, a)] = rho;
    sf[sidx(W_RU0, pos, a)] = r0;
    sf[sidx(W_RU1, pos, a)] = r1;
    sf[sidx(W_RU2, pos, a)] = r2;
    sf[sidx(W_E, pos, a)] = E;
    sf[sidx(W_P, pos, a)] = p;
    sf[sidx(W_A, pos, a)] = sqrt_t(gama * p / rho);
    sf[sidx(W_UD, pos, a)] = DIR == 0 ? u0 : DIR == 1 ? u1 : u2;
  }
  __syncthreads();

  // ---- interface fluxes: interface m of a line sits between cells d0-1+m and d0+m
#pragma unroll 1
  for (int w = 0; w < Tl::IPT; ++w) {
    int m, a;
    if (DIR == 0) { m = tid % TI; a = tid / TI; }
    else { a = tid % TA; m = tid / TA + w * (256 / TA); }
    const int left = d0 - 1 + m;
    if (left <= nd - 1 && a0 + a < na) {
      auto P = [&](int f, int t) -> T { return sf[sidx(f, m + t, a)]; };
      T fl[5];
      interface_flux<T, DIR>(P, gama, eps, fl);
#pragma unroll
      for (int v = 0; v < 5; ++v) sflux[DIR == 0 ? (v * TA + a) * TI + m : (v * TI + m) * TA + a] = fl[v];
    }
  }
  __syncthreads();

  // ---- flux difference for cells d0 .. d0+TI-2
  const T idd = T(ph.inv_delta[DIR]);
  for (int t = tid; t < (TI - 1) * TA; t += 256) {
    int m, a;
    if (DIR == 0) { a = t / (TI - 1); m = t % (TI - 1); }
    else { m = t / TA; a = t % TA; }
    const int c = d0 + m;
    if (c >= nd || a0 + a >= na) continue;
    int i, j, k;
    coords(m + 3, a, i, j, k);
    const int64_t gi = gidx(g, i, j, k);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const T fr = sflux[DIR == 0 ? (v * TA + a) * TI + m + 1 : (v * TI + m + 1) * TA + a];
      const T fl = sflux[DIR == 0 ? (v * TA + a) * TI + m : (v * TI + m) * TA + a];
      const T d = -(fr - fl) * idd;
      if (ACCUM) res.v[v][gi] += d;
      else res.v[v][gi] = d;
    }
  }
}

template <typename T, int DIR, bool ACCUM> static void launch_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r,
                                                                   cudaStream_t s) {
  using Tl = WTile<DIR>;
  const size_t smem = sizeof(T) * ((size_t)W_NF * (Tl::TI + 5) * Tl::TA + 5 * Tl::TI * Tl::TA);
  const int n[3] = {c.g.n0, c.g.n1, c.g.n2};
  const int nt = (n[DIR] + Tl::TI - 2) / (Tl::TI - 1);
  dim3 grid;
  if (DIR == 0) grid = dim3(nt, (n[1] + Tl::TA - 1) / Tl::TA, n[2]);
  else if (DIR == 1) grid = dim3((n[0] + Tl::TA - 1) / Tl::TA, nt, n[2]);
  else grid = dim3((n[0] + Tl::TA - 1) / Tl::TA, n[1], nt);
  k_weno<T, DIR, ACCUM><<<grid, 256, smem, s>>>(c.g, q, r, c.ph);
}

template <typename T>
void launch_weno_dir(const Ctx &c, Fields5<const T> q, Fields5<T> r, int dir, cudaStream_t s, int64_t *launches) {
  if (dir == 0) launch_dir<T, 0, false>(c, q, r, s);
  else if (dir == 1) launch_dir<T, 1, true>(c, q, r, s);
  else launch_dir<T, 2, true>(c, q, r, s);
  ++*launches;
}

template <typename T, int DIR, bool ACCUM> static void attr_dir() {
  using Tl = WTile<DIR>;
  const size_t smem = sizeof(T) * ((size_t)W_NF * (Tl::TI + 5) * Tl::TA + 5 * Tl::TI * Tl::TA);
  cudaFuncSetAttribute(k_weno<T, DIR, ACCUM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
template <typename T> void setup_weno() {
  attr_dir<T, 0, false>();
  attr_dir<T, 1, true>();
  attr_dir<T, 2, true>();
}
template void setup_weno<float>();
template void setup_weno<double>();

template void launch_weno_dir<float>(const Ctx &, Fields5<const float>, Fields5<float>, int, cudaStream_t, int64_t *);
template void launch_weno_dir<double>(const Ctx &, Fields5<const double>, Fields5<double>, int, cudaStream_t,
                                      int64_t *);

}  // namespace osb
