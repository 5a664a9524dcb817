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
//   * WENO5-JS (weno.py:70-205, 341-369): the reference keeps the splitting's factor 1/2 out of f
//     and puts it into the smoothness indicators (1/4 of Jiang-Shu's) and the candidate stencils
//     (1/2 of the usual ones); alpha_r = d_r/(eps + beta_r)^2, omega_r = alpha_r / sum alpha;
//   * flux = REV.(fhat+ + fhat-) (shock_capturing.py:418-448);
//   * residual R -= (flux_{i+1/2} - flux_{i-1/2}) / delta_d.
//
// Arithmetic is rearranged for fewer instructions, not changed in meaning: sqrt(rho_L) u_L is formed
// as rhou_L / sqrt(rho_L); the three dense LEV rows (entropy and both acoustic waves) share one
// dot product g = (phi, -(g-1)u, g-1).X and h = X_{1+d} - u_d X_0 (the flux vector F is never
// stored: its projections are formed from Q, u_d and p):
//     acoustic+- . X = bt (g +- a h),   entropy . X = X_0 - g / a^2;
// the smoothness indicators use Jiang and Shu's sum-of-squares form; the weights take reciprocals
// of (eps+beta)^2 instead of divisions.  In FP32 the reciprocals are the fast hardware ones
// (2 ulp); in FP64 every division is exact.
//
// Tiling: a block covers TA lines along d and computes TI consecutive interfaces per line, giving
// the flux difference of TI-1 cells.  The primitive fields of the TI+5 points of every line sit in
// shared memory (loaded once, coalesced along x).  For y and z each thread owns four consecutive
// interfaces of one line and slides a six-point register window along it, so a point's conserved
// and flux vectors are loaded and formed once per thread instead of six times.
#include "osb_common.cuh"
#include "osb_internal.h"

namespace osb {

namespace {
enum { W_RHO = 0, W_RU0, W_RU1, W_RU2, W_E, W_P, W_A, W_UD, W_NF };

template <int DIR> struct WTile;
template <> struct WTile<0> {  // x: 64 interfaces x 4 rows, one interface per thread
  static constexpr int TI = 64, TA = 4, IPT = 1;
};
template <> struct WTile<1> {  // y: 32 x-lanes x 32 interfaces, four consecutive interfaces per thread
  static constexpr int TI = 32, TA = 32, IPT = 4;
};
template <> struct WTile<2> {
  static constexpr int TI = 32, TA = 32, IPT = 4;
};

template <typename T> __device__ __forceinline__ T rcp_t(T x);
template <> __device__ __forceinline__ float rcp_t<float>(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double rcp_t<double>(double x) { return 1.0 / x; }
template <typename T> __device__ __forceinline__ T rsqrt_t(T x);
template <> __device__ __forceinline__ float rsqrt_t<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_t<double>(double x) { return 1.0 / sqrt(x); }
}  // namespace

// One WENO5-JS side.  f0..f4 are the five stencil values ordered from the far upwind point to the
// far downwind one (for the right-going side: points i-2..i+2; for the left-going side the caller
// passes points i+3..i-1).  d0 weights the most downwind candidate (3/10), d2 the most upwind (1/10).
template <typename T> __device__ __forceinline__ T weno5_side(T f0, T f1, T f2, T f3, T f4, T eps) {
  const T c13 = T(13.0 / 48.0), c14 = T(1.0 / 16.0);
  const T t0 = f2 - T(2) * f3 + f4, s0 = T(3) * f2 - T(4) * f3 + f4;
  const T t1 = f1 - T(2) * f2 + f3, s1 = f1 - f3;
  const T t2 = f0 - T(2) * f1 + f2, s2 = f0 - T(4) * f1 + T(3) * f2;
  const T b0 = c13 * t0 * t0 + c14 * s0 * s0;
  const T b1 = c13 * t1 * t1 + c14 * s1 * s1;
  const T b2 = c13 * t2 * t2 + c14 * s2 * s2;
  const T e0 = b0 + eps, e1 = b1 + eps, e2 = b2 + eps;
  const T a0 = T(3.0 / 10.0) * rcp_t(e0 * e0);
  const T a1 = T(3.0 / 5.0) * rcp_t(e1 * e1);
  const T a2 = T(1.0 / 10.0) * rcp_t(e2 * e2);
  const T p0 = T(1.0 / 6.0) * f2 + T(5.0 / 12.0) * f3 - T(1.0 / 12.0) * f4;
  const T p1 = T(-1.0 / 12.0) * f1 + T(5.0 / 12.0) * f2 + T(1.0 / 6.0) * f3;
  const T p2 = T(1.0 / 6.0) * f0 - T(7.0 / 12.0) * f1 + T(11.0 / 12.0) * f2;
  return (a0 * p0 + a1 * p1 + a2 * p2) * rcp_t(a0 + a1 + a2);
}

// Per-point window entry: conserved vector Q, u_D, a, p.  The physical flux along D,
// F = (Q_{1+D}, Q_{1+c} u_D + delta_cD p, (p + Q_4) u_D), is folded into the projections below.
template <typename T> struct WPt {
  T Q[5], ud, a, p;
};

template <typename T, int D, typename Pt> __device__ __forceinline__ void load_point(const Pt &P, int t, WPt<T> &w) {
  w.Q[0] = P(W_RHO, t);
  w.Q[1] = P(W_RU0, t);
  w.Q[2] = P(W_RU1, t);
  w.Q[3] = P(W_RU2, t);
  w.Q[4] = P(W_E, t);
  w.ud = P(W_UD, t);
  w.p = P(W_P, t);
  w.a = P(W_A, t);
}

// Characteristic flux at the interface between window points 2 and 3 (points i and i+1).
template <typename T, int D>
__device__ __forceinline__ void interface_flux(const WPt<T> (&W)[6], const T gama, const T eps, T out[5]) {
  constexpr int E1 = (D + 1) % 3, E2 = (D + 2) % 3;  // the two tangential axes (shear rows)
  constexpr int e1 = 3 - E1 - D, e2 = 3 - E2 - D;    // third axis of each shear row
  const T gm1 = gama - T(1);
  // ---- Roe average of points 2 and 3
  const T rl = W[2].Q[0], rr = W[3].Q[0];
  const T isl = rsqrt_t(rl), isr = rsqrt_t(rr);  // 1/sqrt(rho)
  const T sl = rl * isl, sr = rr * isr;          // sqrt(rho)
  const T rho = sl * sr;
  const T inv_s = rcp_t(sl + sr);
  T u[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = inv_s * (W[2].Q[1 + c] * isl + W[3].Q[1 + c] * isr);
  const T Hh = inv_s * ((W[2].p + W[2].Q[4]) * isl + (W[3].p + W[3].Q[4]) * isr);
  const T usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const T a = sqrt_t(gm1 * (Hh - T(0.5) * usq));
  const T ia = rcp_t(a), irho = rcp_t(rho);
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
  auto recon = [&](const T (&cf)[6], const T (&cs)[6], T lam) -> T {
    T fp[6], fm[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      fp[t] = cf[t] + lam * cs[t];
      fm[t] = cf[t] - lam * cs[t];
    }
    return weno5_side(fp[0], fp[1], fp[2], fp[3], fp[4], eps) + weno5_side(fm[5], fm[4], fm[3], fm[2], fm[1], eps);
  };

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
  const T igm1 = rcp_t(gm1);
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

template <typename T, int DIR, bool ACCUM>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) k_weno(Grid g, Fields5<const T> q, Fields5<T> res, Phys ph) {
  using Tl = WTile<DIR>;
  constexpr int TI = Tl::TI, TA = Tl::TA, NPT = TI + 5;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sf = reinterpret_cast<T *>(smem_raw);   // [W_NF][NPT][TA] (DIR>0) or [W_NF][TA][NPT] (DIR==0)
  T *sflux = sf + W_NF * NPT * TA;           // [5][TI][TA] or [5][TA][TI]
  const int tid = threadIdx.x;
  const int n[3] = {g.n0, g.n1, g.n2};
  const T gm1 = pick<T>(ph.gm1, ph.f_gm1), gama = pick<T>(ph.gama, ph.f_gama);
  const T eps = pick<T>(ph.weno_eps, ph.f_eps);

  // tile origin: first cell whose flux difference this block writes (d0), across-line origin
  int d0, a0, o1, o2;
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
    const T irho = T(1) / rho;
    const T u0 = r0 * irho, u1 = r1 * irho, u2 = r2 * irho;
    const T half = T(0.5);
    const T p = gm1 * (E - half * rho * u0 * u0 - half * rho * u1 * u1 - half * rho * u2 * u2);
    sf[sidx(W_RHO, pos, a)] = rho;
    sf[sidx(W_RU0, pos, a)] = r0;
    sf[sidx(W_RU1, pos, a)] = r1;
    sf[sidx(W_RU2, pos, a)] = r2;
    sf[sidx(W_E, pos, a)] = E;
    sf[sidx(W_P, pos, a)] = p;
    sf[sidx(W_A, pos, a)] = sqrt_t(gama * p * irho);
    sf[sidx(W_UD, pos, a)] = DIR == 0 ? u0 : DIR == 1 ? u1 : u2;
  }
  __syncthreads();

  // ---- interface fluxes: interface m of a line sits between cells d0-1+m and d0+m and uses the
  //      points at positions m..m+5
  auto flux_store = [&](int m, int a, const T (&fl)[5]) {
#pragma unroll
    for (int v = 0; v < 5; ++v) sflux[DIR == 0 ? (v * TA + a) * TI + m : (v * TI + m) * TA + a] = fl[v];
  };
  if (DIR == 0) {
    const int m = tid % TI, a = tid / TI;
    if (d0 - 1 + m <= nd - 1 && a0 + a < na) {
      auto P = [&](int f, int t) -> T { return sf[sidx(f, m + t, a)]; };
      WPt<T> W[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) load_point<T, DIR>(P, t, W[t]);
      T fl[5];
      interface_flux<T, DIR>(W, gama, eps, fl);
      flux_store(m, a, fl);
    }
  } else {
    const int a = tid % TA, m0 = (tid / TA) * Tl::IPT;
    auto P = [&](int f, int t) -> T { return sf[sidx(f, m0 + t, a)]; };
    if (a0 + a < na && d0 - 1 + m0 <= nd - 1) {
      WPt<T> W[6];
#pragma unroll
      for (int t = 0; t < 5; ++t) load_point<T, DIR>(P, t, W[t]);
#pragma unroll 1
      for (int w = 0; w < Tl::IPT; ++w) {
        if (d0 - 1 + m0 + w <= nd - 1) {
          load_point<T, DIR>(P, w + 5, W[5]);
          T fl[5];
          interface_flux<T, DIR>(W, gama, eps, fl);
          flux_store(m0 + w, a, fl);
        }
#pragma unroll
        for (int t = 0; t < 5; ++t) W[t] = W[t + 1];
      }
    }
  }
  __syncthreads();

  // ---- flux difference for cells d0 .. d0+TI-2
  const T idd = pick<T>(ph.inv_delta[DIR], ph.f_inv_delta[DIR]);
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
